"""Centroid trace of the multi-turn wake workload at full size, for the
growth-rate parity test (tests/test_gpu_growth_full.py):

    python tests/golden/make_golden_c3_growth.py --ref <PyHEADTAIL tree>
    python tests/golden/make_golden_c3_growth.py --impl oracle [--save F]

Workload: 1e7 macroparticles (numpy seed 2, the reference generator's draw
order), gamma 27.7, one smooth transverse segment (Q 20.13 / 20.18, beta
50 m, Q' = 0), RF h = 4620, V = 4.5 MV, UniformBinSlicer(500, z_cuts=(-0.69,
0.69)), CircularResonator(10 MOhm/m, 1 GHz, Q = 1) and
CircularResistiveWall(20 mm, 6911.5 m, 5.8e7 S/m, dt_min 1e-12, 50 turns),
2000 turns.  The turn loop is the reference test's
(tests/simulation_tests/test_bb_resonator.py:91-96: every element's track,
then bunch.mean_x(), bunch.mean_y()).

--impl reference (the default) runs PyHEADTAIL itself (copied to a scratch
directory and its Cython module built there) and writes
tests/golden/growth/c3_1e7.npz with mean_x, mean_y of every turn and the
growth rates of the reference test's method (Hilbert envelope, linear fit
of its logarithm) over the second half of the run.  --impl oracle runs the
NumPy oracle on the same bunch; when the reference's file exists it prints
how far the two traces are apart, and --save keeps the oracle's trace.
Each run takes of the order of an hour on one core.
"""
import argparse
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, HERE)
sys.path.insert(0, ROOT)
import cases as C  # noqa: E402

N_PART, SEED, N_TURNS, N_SLICES, RW_TURNS = 10000000, 2, 2000, 500, 50
OUT = os.path.join(HERE, 'growth', 'c3_1e7.npz')


def spec():
    return dict(beam=C.beam_params(N_PART, SEED), n_turns=N_TURNS,
                elements=[C.smooth_transverse(), C.rf(),
                          C.wake(C.slicer(N_SLICES), C.resonator(),
                                 C.resistive_wall(n_turns_wake=RW_TURNS))])


def growth_rate(centroid, first=N_TURNS // 2):
    """The reference test's fit (test_bb_resonator.py:99-106) over turns
    [first, end)."""
    from scipy.signal import hilbert
    from scipy.stats import linregress
    env = np.abs(hilbert(centroid))
    turns = np.arange(len(centroid))
    return linregress(turns[first:], np.log(env[first:]))[0]


def run_reference(ref, scratch):
    import make_golden as MG
    MG.build_reference(ref, scratch)
    sp = spec()
    beam = MG.make_beam(sp['beam'])
    elements = [el for _, el in MG.make_elements(sp, beam)]
    return beam, elements


def run_oracle():
    from oracle import cases as OC
    sp = spec()
    beam = OC.make_beam(sp['beam'])
    elements = [el for _, el in OC.make_elements(sp, beam)]
    return beam, elements


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('--impl', choices=['reference', 'oracle'],
                    default='reference')
    ap.add_argument('--ref', help='PyHEADTAIL source tree (read only)')
    ap.add_argument('--scratch', default='/tmp/phk_refbuild')
    ap.add_argument('--save', help='oracle: write its trace to this .npz')
    a = ap.parse_args()
    if a.impl == 'reference':
        if not a.ref:
            ap.error('--ref is required with --impl reference')
        beam, elements = run_reference(a.ref, a.scratch)
    else:
        beam, elements = run_oracle()
    mx = np.zeros(N_TURNS)
    my = np.zeros(N_TURNS)
    t0 = time.time()
    for i in range(N_TURNS):
        for el in elements:
            el.track(beam)
        mx[i], my[i] = beam.mean_x(), beam.mean_y()
        if i % 100 == 0:
            print('turn %d  %.1f s  mean_x %.6e' % (i, time.time() - t0,
                                                    mx[i]), flush=True)
    gx, gy = growth_rate(mx), growth_rate(my)
    print('%s growth rate x %.6e y %.6e per turn' % (a.impl, gx, gy))
    if a.impl == 'reference':
        os.makedirs(os.path.dirname(OUT), exist_ok=True)
        np.savez_compressed(OUT, mean_x=mx, mean_y=my, growth_x=gx,
                            growth_y=gy, n_macroparticles=N_PART, seed=SEED,
                            n_slices=N_SLICES, rw_turns=RW_TURNS)
        print('wrote', OUT)
    elif a.save:
        np.savez_compressed(a.save, mean_x=mx, mean_y=my, growth_x=gx,
                            growth_y=gy)
    if a.impl == 'oracle' and os.path.exists(OUT):
        f = np.load(OUT)
        for q, o in (('mean_x', mx), ('mean_y', my)):
            r = f[q]
            print('%s: oracle - reference max %.3e (trace rms %.3e)' % (
                q, np.max(np.abs(o - r)), np.sqrt(np.mean(r**2))))
        print('growth x %.6e vs %.6e, y %.6e vs %.6e' % (
            gx, float(f['growth_x']), gy, float(f['growth_y'])))


if __name__ == '__main__':
    main()
