"""Host-side API of the path's element classes (no GPU): the chromaticity
polynomials a ChromaticitySegment exposes (calc_detuning_x / _y and
_make_calc_detuning, detuners.py:48-98) against the oracle's restatement,
including the reference's order > 3 behaviour (one more zero coefficient
prepended on every call, detuners.py:95-97) and its agreement with what the
kernel is told (_pack); RFSystems' removed-interface notices and
clean_buckets (longitudinal_tracking.py:525-648); LinearMap.Qs (:716-718)."""
import numpy as np
import pytest
from scipy.constants import e, m_p

from oracle import turn_loop as T

from pyheadtail_gb300.trackers.detuners import ChromaticitySegment
from pyheadtail_gb300.trackers.longitudinal_tracking import (LinearMap,
                                                             RFSystems)


@pytest.mark.parametrize('qp_x,qp_y', [([5.], [-3.]), ([3., 120.], [1.5]),
                                       ([-2., 40., 9000.], [7., 0., 1e4]),
                                       ([1., 2., 3., 4., 5.], [2.]),
                                       ([0.5, 1., 2., 3.], [1., 2., 3., 4.])])
def test_chromaticity_polynomials_match_oracle(qp_x, qp_y):
    rng = np.random.RandomState(4)
    seg = ChromaticitySegment(qp_x, qp_y)
    ref = T.ChromaDetuner(qp_x, qp_y)
    standalone = ChromaticitySegment._make_calc_detuning(np.atleast_1d(qp_x))
    ref_alone = T.ChromaDetuner(qp_x, qp_y)
    for call in range(3):
        dp = rng.normal(0, 1e-3, 1000)
        np.testing.assert_array_equal(seg.calc_detuning_x(dp),
                                      ref._poly(ref.cx, dp))
        np.testing.assert_array_equal(seg.calc_detuning_y(dp),
                                      ref._poly(ref.cy, dp))
        np.testing.assert_array_equal(standalone(dp),
                                      ref_alone._poly(ref_alone.cx, dp))
    # the kernel sees the same number of prepended zeros as the host
    # polynomials have reached (one more call)
    pack = seg._pack(None)
    ref._poly(ref.cx, dp)
    ref._poly(ref.cy, dp)
    for n, z, cs in ((pack.nx, pack.zx, ref.cx), (pack.ny, pack.zy, ref.cy)):
        if n > 3:
            assert z == len(cs) - n - 1
        else:
            assert z == 0


def _rf():
    return RFSystems(6911.5, [4620, 9240], [4.5e6, 0.45e6], [0., 0.],
                     [1.8e-3], 27.7, charge=e, mass=m_p)


@pytest.mark.parametrize('name', ['rfbucket', 'kicks', 'elements',
                                  'fundamental_kick', 'accelerating_kick'])
def test_rfsystems_removed_attributes_raise_as_reference(name):
    with pytest.raises(RuntimeError, match='Interface change'):
        getattr(_rf(), name)


@pytest.mark.parametrize('name', ['set_voltage_list', 'set_harmonic_list',
                                  'set_phi_offset_list'])
def test_rfsystems_removed_setters_raise_as_reference(name):
    with pytest.raises(RuntimeError, match='Interface change'):
        getattr(_rf(), name)([1.])


def test_rfsystems_lists_and_buckets_still_work():
    rf = _rf()
    assert list(rf.voltages) == [4.5e6, 0.45e6]
    assert list(rf.harmonics) == [4620, 9240]
    rf.clean_buckets()
    assert rf._rfbuckets == {}


def test_linear_map_qs():
    lm = LinearMap([1.8e-3], 6911.5, 0.017)
    assert lm.Qs == lm.Q_s == 0.017
