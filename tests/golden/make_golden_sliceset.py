"""Golden values of the reference's SliceSet analysis methods
(particles/slicing.py:133-292: smoothing_sigma, particle_indices_by_slice,
pidx_begin / pidx_end, lambda_bins, lambda_prime_bins, lambda_z,
lambda_prime_z), made by running PyHEADTAIL itself on a seeded bunch:

    python tests/golden/make_golden_sliceset.py --ref <PyHEADTAIL source tree>

Writes tests/golden/sliceset/analysis.npz (a subdirectory, apart from
the turn-loop fixtures that the parity tests collect): the slicing (z_bins, slice index
of every particle, counts, charge per macroparticle) and every method's
output, for a uniform-bin and a uniform-charge slicing.
"""
import argparse
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import cases as C  # noqa: E402
import make_golden as MG  # noqa: E402


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('--ref', required=True,
                    help='PyHEADTAIL source tree (read only)')
    ap.add_argument('--scratch', default='/tmp/pyht_ref')
    a = ap.parse_args()
    MG.build_reference(a.ref, a.scratch)
    MG.patch_reference_numpy2()
    from PyHEADTAIL.particles.slicing import (UniformBinSlicer,
                                              UniformChargeSlicer,
                                              ModeIsUniformCharge)
    beam = MG.make_beam(C.beam_params(4000, 41))
    zq = np.linspace(-0.8, 0.8, 97)
    out = {}
    for tag, slicer in (('bin', UniformBinSlicer(64, z_cuts=(-0.69, 0.69))),
                        ('charge', UniformChargeSlicer(48, n_sigma_z=3))):
        ss = slicer.slice(beam)
        p = tag + '_'
        out[p + 'z_bins'] = np.asarray(ss.z_bins, dtype=np.float64)
        out[p + 'idx'] = np.asarray(ss.slice_index_of_particle, np.int32)
        out[p + 'counts'] = np.asarray(ss.n_macroparticles_per_slice,
                                       np.int32)
        out[p + 'charge_per_mp'] = np.float64(ss.charge_per_mp)
        out[p + 'mode'] = np.array(ss.mode)
        out[p + 'smoothing_sigma'] = np.float64(ss.smoothing_sigma)
        out[p + 'by_slice'] = np.asarray(ss.particle_indices_by_slice,
                                         np.int64)
        out[p + 'pidx_begin'] = np.int64(ss.pidx_begin)
        out[p + 'pidx_end'] = np.int64(ss.pidx_end)
        out[p + 'within'] = np.asarray(ss.particles_within_cuts_slice,
                                       np.int64)
        out[p + 'lambda_bins'] = ss.lambda_bins()
        out[p + 'lambda_bins_raw'] = ss.lambda_bins(sigma=3., smoothen=False)
        out[p + 'lambda_z'] = ss.lambda_z()
        out[p + 'lambda_zq'] = ss.lambda_z(zq)
        try:
            out[p + 'lambda_prime_bins'] = ss.lambda_prime_bins()
            out[p + 'lambda_prime_bins_s2'] = ss.lambda_prime_bins(
                sigma=2., smoothen_before=False)
            out[p + 'lambda_prime_zq'] = ss.lambda_prime_z(zq)
        except ModeIsUniformCharge:
            out[p + 'lambda_prime_raises'] = np.bool_(True)
    out['zq'] = zq
    path = os.path.join(HERE, 'sliceset', 'analysis.npz')
    np.savez_compressed(path, **out)
    print('wrote', path, len(out), 'arrays')


if __name__ == '__main__':
    main()
