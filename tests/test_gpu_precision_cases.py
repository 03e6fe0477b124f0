"""The FP32 precision form on every golden case: each fixture's element
sequence (transverse maps with dispersion and detuning, RF with several
harmonics or acceleration, linear maps, resonator / plates / multi-turn /
table wakes, uniform-charge slicing, dampers) runs in the precision form
from the fixture's initial bunch rounded to FP32, against the FP64 oracle
run from the same rounded bunch.  The difference is then the form's own
arithmetic: coordinates stored in FP32 every turn, float-float phases,
FP32 slice sums.  Bars: the RMS over particles of the error relative to the
coordinate's RMS, and the beam's scalars (gamma, p0), which the form keeps
in FP64 on the host, bit for bit.

Measured on a GB300: 1e-7 (the FP32 rounding) on most cases; up to 1.8e-4
where strong amplitude detuning turns the per-turn rounding of x, xp into
phase errors (c2_full; transverse_segments_dispersion, whose detuning
reaches 1.2 turns: a float32 emulation of the map on the host gives the
same 1.2e-4 on xp).  The bar is five times the largest."""
import glob
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip('torch')

GOLDEN = os.path.join(os.path.dirname(__file__), 'golden')
FIXTURES = sorted(p for p in glob.glob(os.path.join(GOLDEN, '*.npz'))
                  if 'spec' in np.load(p).files)
COORDS = ('x', 'xp', 'y', 'yp', 'z', 'dp')
RMS_BAR = 1e-3


@pytest.mark.parametrize('path', FIXTURES,
                         ids=[os.path.basename(p)[:-4] for p in FIXTURES])
def test_golden_case_in_fp32_form(path):
    import gpu_cases as G
    from oracle import cases as OC
    with np.load(path) as f:
        spec = json.loads(str(f['spec']))
        coords = {k: f['init_' + k].astype(np.float32).astype(np.float64)
                  for k in COORDS}
    n_turns = spec['n_turns']
    last = n_turns - 1
    ob = OC.make_beam(spec['beam'], coords)
    ref = OC.run(spec, ob, n_turns=n_turns, record_turns=(last,))
    beam = G.make_beam(spec['beam'], coords, precision='fp32')
    rec = G.run(spec, beam, n_turns=n_turns, record_turns=(last,))
    errs = {}
    for q in COORDS:
        r = np.asarray(ref['t%d_%s' % (last, q)], np.float64)
        g = np.asarray(rec['t%d_%s' % (last, q)], np.float64)
        scale = np.sqrt(np.mean(r**2)) or 1.
        errs[q] = float(np.sqrt(np.mean(((g - r) / scale)**2)))
    print('%s fp32 form, %d turns: %s' % (
        os.path.basename(path), n_turns,
        ' '.join('%s %.2e' % kv for kv in errs.items())))
    for q, e in errs.items():
        assert e <= RMS_BAR, (q, e)
    for k in ('gamma', 'p0'):
        key = 't%d_%s' % (last, k)
        if key in ref:
            assert float(rec[key]) == float(ref[key]), (k, rec[key], ref[key])
