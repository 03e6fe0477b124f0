"""Host-side API of the path's element classes (no GPU): the chromaticity
polynomials a ChromaticitySegment exposes (calc_detuning_x / _y and
_make_calc_detuning, detuners.py:48-98) against the oracle's restatement,
including the reference's order > 3 behaviour (one more zero coefficient
prepended on every call, detuners.py:95-97) and its agreement with what the
kernel is told (_pack); RFSystems' removed-interface notices and
clean_buckets (longitudinal_tracking.py:525-648); LinearMap.Qs (:716-718);
the dispersion entry points of Kick and LinearMap (:183-203, :731-759)."""
import numpy as np
import pytest
from scipy.constants import c, e, m_p

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


class _LongBeam(object):
    """The beam scalars and engine that Kick / LinearMap ops read."""

    def __init__(self):
        self.charge, self.mass = e, m_p
        self.gamma = 27.7
        self.beta = np.sqrt(1 - self.gamma**-2)
        self.p0 = np.sqrt(self.gamma**2 - 1) * m_p * c
        self.ops = []
        beam = self

        class _Engine(object):
            def enqueue(self, op):
                beam.ops.append(op)
        self._engine = _Engine()

    def clean_slices(self):
        pass


@pytest.mark.parametrize('D', [0., 0.7])
def test_dispersion_entry_points(D):
    """track follows D_x, D_y (the reference binds track to one of the two);
    track_with_dispersion / track_without_dispersion set or clear the
    dispersion passes whatever D is, with all other parameters equal."""
    from pyheadtail_gb300 import _native as N
    from pyheadtail_gb300.trackers.longitudinal_tracking import Kick
    for el in (Kick([1.8e-3], 6911.5, 4620, 4.5e6, D_x=D),
               LinearMap([1.8e-3], 6911.5, 0.017, D_x=D)):
        ops = {}
        for m in ('track', 'track_with_dispersion', 'track_without_dispersion'):
            b = _LongBeam()
            getattr(el, m)(b)
            ops[m] = b.ops[0]
        disp = {m: bool(op.flags & N.FLAG_DISPERSION) for m, op in ops.items()}
        assert disp == {'track': D != 0, 'track_with_dispersion': True,
                        'track_without_dispersion': False}
        for op in ops.values():
            assert op.p == ops['track'].p and op.kind == ops['track'].kind
            assert (op.flags | N.FLAG_DISPERSION) == \
                (ops['track'].flags | N.FLAG_DISPERSION)
