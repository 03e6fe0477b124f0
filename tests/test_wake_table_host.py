"""WakeTable on the host (no GPU): the sampled wake functions, the kick
list and the input checks agree with the oracle's restatement, which the
wake_table_* fixtures pin to the reference."""
import os

import numpy as np
import pytest

from oracle import turn_loop as T

pytest.importorskip('torch')

from pyheadtail_gb300.general.printers import SilentPrinter  # noqa: E402
from pyheadtail_gb300.impedances import wakes as W  # noqa: E402
from pyheadtail_gb300.particles.slicing import UniformBinSlicer  # noqa: E402

GOLDEN = os.path.join(os.path.dirname(__file__), 'golden')
COLS = ['time', 'constant_x', 'dipole_x', 'dipole_y', 'dipole_xy',
        'dipole_yx', 'quadrupole_x', 'quadrupole_y', 'longitudinal']


@pytest.mark.parametrize('name', ['wake_table_ultra.dat',
                                  'wake_table_lowbeta.dat'])
def test_functions_and_kicks_match_oracle(name):
    path = os.path.join(GOLDEN, name)
    wt = W.WakeTable(path, COLS, n_turns_wake=1, printer=SilentPrinter())
    table = T.load_wake_table(path, COLS)
    rng = np.random.RandomState(1)
    dt = -rng.uniform(0, 4.5e-9, 2000)
    if name.endswith('lowbeta.dat'):
        dt = rng.uniform(-4.5e-9, 4.5e-9, 2000)
    for comp in COLS[1:-1]:
        np.testing.assert_array_equal(wt.function_transverse(comp)(dt),
                                      T.table_transverse(table, comp)(dt))
    np.testing.assert_array_equal(wt.function_longitudinal()(dt),
                                  T.table_longitudinal(table)(dt))
    sl = UniformBinSlicer(20, z_cuts=(-0.5, 0.5), warningprinter=SilentPrinter())
    kicks = wt.get_wake_kicks(sl)
    want = [(t, m, q) for c, t, m, q in T.TABLE_KICKS if c in COLS]
    got = [(k.target, None if k.moment == 'count' else k.moment, k.quad)
           for k in kicks]
    assert got == want


def test_input_checks(tmp_path):
    path = os.path.join(GOLDEN, 'wake_table_ultra.dat')
    with pytest.raises(ValueError):
        W.WakeTable(path, COLS[:-1])
    with pytest.raises(ValueError):
        W.WakeTable(path, ['t'] + COLS[1:])
    bad = np.loadtxt(path)
    bad[:, 0] += 1.0            # starts after 0: neither branch applies
    p = str(tmp_path / 'late.dat')
    np.savetxt(p, bad)
    wt = W.WakeTable(p, COLS, printer=SilentPrinter())
    with pytest.raises(ValueError):
        wt.function_transverse('dipole_x')
    # ultrarelativistic transverse samples beyond the table raise
    wt = W.WakeTable(path, COLS, printer=SilentPrinter())
    with pytest.raises(ValueError):
        wt.function_transverse('dipole_x')(np.array([-1.0]))
