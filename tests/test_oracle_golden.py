"""Pin the CPU oracle against fixtures made by running the PyHEADTAIL
reference (tests/golden/make_golden.py).

The oracle restates the reference's NumPy/Cython arithmetic in the same
operation order, so everything is compared bit for bit: coordinates, beam
scalars, slice indices, counts, bins, per-slice statistics and every bunch
statistic of Particles (``bunch_statistics``).
"""
import glob
import json
import os

import numpy as np
import pytest

from oracle import cases as OC
from oracle import turn_loop as T

GOLDEN = os.path.join(os.path.dirname(__file__), 'golden')
FIXTURES = sorted(glob.glob(os.path.join(GOLDEN, '*.npz')))


def load(path):
    with np.load(path) as f:
        return {k: f[k] for k in f.files}


@pytest.mark.parametrize('path', FIXTURES,
                         ids=[os.path.basename(p)[:-4] for p in FIXTURES])
def test_oracle_matches_reference_bit_for_bit(path):
    g = load(path)
    spec = json.loads(str(g['spec']))
    # the bunch itself: the oracle's generator restatement must reproduce
    # the reference generator's seeded draw exactly
    beam = OC.make_beam(spec['beam'])
    for k in T.Beam.COORDS:
        np.testing.assert_array_equal(getattr(beam, k), g['init_' + k],
                                      err_msg='generator ' + k)
    rec = OC.run(spec, beam)
    keys = [k for k in g if k.startswith('t')]
    assert keys
    for k in keys:
        assert k in rec, k
        np.testing.assert_array_equal(rec[k], g[k], err_msg=k)


def test_fixture_set_covers_every_stage():
    names = {os.path.basename(p)[:-4] for p in FIXTURES}
    for need in ('transverse_chroma_amp', 'transverse_segments_dispersion',
                 'linear_map', 'rf_double_harmonic', 'rf_accelerating',
                 'slicer_fixed', 'wake_resonator', 'wake_multiturn',
                 'wake_dynamic_cuts', 'wake_plates', 'c1_full', 'c2_full',
                 'c3_full', 'c5_full',
                 'bunch_statistics', 'wake_table_multiturn',
                 'wake_table_lowbeta', 'damper_resistive',
                 'damper_reactive', 'charge_slicer', 'wake_charge_slicer'):
        assert need in names
