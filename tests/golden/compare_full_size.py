"""Run the PyHEADTAIL reference itself and the oracle side by side at a
workload's full size: time one core of each, and check that every
coordinate is bit-identical after the same turns.

Run in a container where the reference source tree is present (built in a
scratch directory as make_golden.py does):

    python tests/golden/compare_full_size.py --ref <PyHEADTAIL source tree> \\
        --workload c3 --turns 3

Workloads: c3 -- 1e7 macroparticles, 500 slices, resonator + 50-turn
resistive wall, RF h=4620; c5 -- 5e7 macroparticles, Q' 2, amplitude
detuning, 1000 slices, the same wakes.  The bunch is drawn with the
reference's own generator and handed to the oracle as coordinates.  One
untimed turn precedes the timed ones.  Single-threaded BLAS is advised
(OMP_NUM_THREADS=1): the reference is a single-core NumPy code.
"""
import argparse
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
import cases as C  # noqa: E402
import make_golden as MG  # noqa: E402

AMP = [1e-11, 1e-11, -5e-12]
WORKLOADS = {
    'c3': dict(n=10**7, seed=2, slices=500, chroma=None, amp=None),
    'c5': dict(n=5 * 10**7, seed=4, slices=1000, chroma=[2., 2.], amp=AMP),
}
COORDS = ('x', 'xp', 'y', 'yp', 'z', 'dp')


def spec_of(w, n, turns):
    return dict(beam=C.beam_params(n, w['seed']), n_turns=turns, elements=[
        C.smooth_transverse(chroma=w['chroma'], amplitude=w['amp']), C.rf(),
        C.wake(C.slicer(w['slices']), C.resonator(),
               C.resistive_wall(n_turns_wake=50))])


def timed(elements, beam, turns):
    for m in elements:                  # untimed first turn
        m.track(beam)
    t0 = time.perf_counter()
    for _ in range(turns):
        for m in elements:
            m.track(beam)
    return (time.perf_counter() - t0) / turns


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('--ref', required=True,
                    help='PyHEADTAIL source tree (read only)')
    ap.add_argument('--scratch', default='/tmp/phk_refbuild')
    ap.add_argument('--workload', choices=sorted(WORKLOADS), default='c3')
    ap.add_argument('--n', type=int, default=None,
                    help='macroparticles (default: the workload size)')
    ap.add_argument('--turns', type=int, default=3)
    a = ap.parse_args()
    MG.build_reference(a.ref, a.scratch)
    MG.patch_reference_numpy2()
    from oracle import cases as OC
    w = WORKLOADS[a.workload]
    n = a.n or w['n']
    spec = spec_of(w, n, a.turns)

    ref_beam = MG.make_beam(spec['beam'])
    coords = {k: getattr(ref_beam, k).copy() for k in COORDS}
    ref_elements = [el for _, el in MG.make_elements(spec, ref_beam)]
    t_ref = timed(ref_elements, ref_beam, a.turns)

    oracle_beam = OC.make_beam(spec['beam'], coords)
    oracle_elements = [el for _, el in OC.make_elements(spec, oracle_beam)]
    t_oracle = timed(oracle_elements, oracle_beam, a.turns)

    same = {k: bool(np.array_equal(getattr(ref_beam, k),
                                   getattr(oracle_beam, k))) for k in COORDS}
    print('%s, %d macroparticles, %d turns' % (a.workload, n, a.turns + 1))
    print('reference: %.3f s per turn, %.3g macroparticle-turns/s'
          % (t_ref, n / t_ref))
    print('oracle:    %.3f s per turn, %.3g macroparticle-turns/s'
          % (t_oracle, n / t_oracle))
    print('bit-identical coordinates:', same)
    if not all(same.values()):
        sys.exit(1)


if __name__ == '__main__':
    main()
