"""Bunch statistics from one record of ``phk_bunch_stats``.

PyHEADTAIL computes each statistic of a bunch with its own pass over the
particles (particles/particles.py:311-390 through general/pmath.py:183-189:
``np.mean`` and the Cython functions of cobra_functions/stats.pyx).  Its
covariance is a shifted single pass with the shift a[0] (stats.pyx:17-45):

    cov(a, b) = (S_ab - S_a * S_b / n) / (n - 1),
    S_a = sum_i (a_i - a_0),   S_ab = sum_i (a_i - a_0) (b_i - b_0).

One device pass (``phk_bunch_stats``) produces n, the shifts, every S_a
and the 13 S_ab that some statistic uses (order 2; an order-1 record holds
plain sums with shift 0); every statistic below is the reference's formula
evaluated on those sums in FP64:

* mean_q = a_0 + S_q / n (the reference's np.mean sums pairwise, so the
  two agree to rounding, not bit for bit);
* cov, std, emittance, get_alpha / get_beta / get_gamma as stats.pyx:49-185;
* dispersion = <u dp> / <dp^2> (stats.pyx:57-70) with the raw moments
  recovered from the shifted sums.
"""
import numpy as np

COORDS = ('x', 'xp', 'y', 'yp', 'z', 'dp')
INDEX = {k: i for i, k in enumerate(COORDS)}
RECORD_LEN = 34

# record entry of the pair sum S_ab, a <= b, in the order of the record
_PAIR = {}
_p = 13
for _a in range(6):
    for _b in range(_a, 6):
        _PAIR[(_a, _b)] = _PAIR[(_b, _a)] = _p
        _p += 1
del _p, _a, _b

# the pair sums an order-2 record holds (the others are written as 0)
USED_PAIRS = [('x', 'x'), ('x', 'xp'), ('xp', 'xp'), ('y', 'y'), ('y', 'yp'),
              ('yp', 'yp'), ('z', 'z'), ('z', 'dp'), ('dp', 'dp'),
              ('x', 'dp'), ('xp', 'dp'), ('y', 'dp'), ('yp', 'dp')]

# the coordinates and the order (1: first sums, 2: pair sums) each
# statistic of Particles needs
_U = {'x': ('x', 'xp'), 'y': ('y', 'yp')}
NEEDS = {}
for _q in COORDS:
    NEEDS['mean_' + _q] = ((_q,), 1)
    NEEDS['sigma_' + _q] = ((_q,), 2)
for _pl in ('x', 'y'):
    NEEDS['effective_normalized_emittance_' + _pl] = (_U[_pl], 2)
    NEEDS['epsn_' + _pl] = (_U[_pl] + ('dp',), 2)
    NEEDS['dispersion_' + _pl] = ((_pl, 'dp'), 2)
    for _tw in ('alpha', 'beta', 'gamma'):
        NEEDS['%s_Twiss_%s' % (_tw, _pl)] = (_U[_pl] + ('dp',), 2)
NEEDS['effective_normalized_emittance_z'] = (('z', 'dp'), 2)
NEEDS['epsn_z'] = (('z', 'dp'), 2)
del _q, _pl, _tw


def mask_of(coords):
    m = 0
    for q in coords:
        m |= 1 << INDEX[q]
    return m


class StatsRecord(object):
    """The sums of one bunch state and the statistics derived from them."""

    def __init__(self, record, mask=0x3f, order=2):
        r = np.asarray(record, dtype=np.float64)
        if r.shape != (RECORD_LEN,):
            raise ValueError('a statistics record has %d entries' % RECORD_LEN)
        self.r = r
        self.n = int(r[0])
        self.mask = mask
        self.order = order

    def covers(self, coords, order):
        m = mask_of(coords)
        return order <= self.order and (self.mask & m) == m

    # -- sums
    def _s1(self, q):
        return self.r[7 + INDEX[q]]

    def _s2(self, a, b):
        return self.r[_PAIR[(INDEX[a], INDEX[b])]]

    def _shift(self, q):
        return self.r[1 + INDEX[q]]

    # -- the reference's statistics
    def mean(self, q):
        if self.n == 0:
            return np.nan
        return self._shift(q) + self._s1(q) / self.n

    def cov(self, a, b):
        """stats.pyx:17-45."""
        n = self.n
        if n < 2:
            return 0.
        return (self._s2(a, b) - self._s1(a) * self._s1(b) / n) / (n - 1)

    def std(self, q):
        """stats.pyx:49-54."""
        return np.sqrt(self.cov(q, q))

    def dispersion(self, u, dp='dp'):
        """stats.pyx:57-70."""
        n = self.n
        su, sd = self._shift(u), self._shift(dp)
        s_u, s_d = self._s1(u), self._s1(dp)
        mean_u_dp = (self._s2(u, dp) + sd * s_u + su * s_d + n * su * sd) / n
        mean_dp2 = (self._s2(dp, dp) + 2 * sd * s_d + n * sd * sd) / n
        if mean_dp2 > 0:
            return mean_u_dp / mean_dp2
        return 0

    def emittance(self, u, up, dp):
        """stats.pyx:73-122 (dp None: the effective emittance)."""
        cov_u2 = self.cov(u, u)
        cov_up2 = self.cov(up, up)
        cov_u_up = self.cov(up, u)
        t11 = t12 = t22 = 0.
        if dp is not None:
            cov_dp2 = self.cov(dp, dp)
            if cov_dp2 != 0:
                cov_u_dp = self.cov(u, dp)
                cov_up_dp = self.cov(up, dp)
                t11 = cov_u_dp * cov_u_dp / cov_dp2
                t12 = cov_u_dp * cov_up_dp / cov_dp2
                t22 = cov_up_dp * cov_up_dp / cov_dp2
        s11, s12, s22 = cov_u2 - t11, cov_u_up - t12, cov_up2 - t22
        return np.sqrt(s11 * s22 - s12 * s12)

    def _twiss_terms(self, u, up, dp):
        if dp is None:
            return 1., 0., 0.
        return self.cov(dp, dp), self.cov(u, dp), self.cov(up, dp)

    def alpha(self, u, up, dp):
        """stats.pyx:126-145."""
        cov_dp2, cov_u_dp, cov_up_dp = self._twiss_terms(u, up, dp)
        sigma12 = self.cov(u, up) - cov_u_dp * cov_up_dp / cov_dp2
        return -sigma12 / self.emittance(u, up, dp)

    def beta(self, u, up, dp):
        """stats.pyx:148-165."""
        cov_dp2, cov_u_dp, _ = self._twiss_terms(u, up, dp)
        sigma11 = self.cov(u, u) - cov_u_dp * cov_u_dp / cov_dp2
        return sigma11 / self.emittance(u, up, dp)

    def gamma(self, u, up, dp):
        """stats.pyx:168-185."""
        cov_dp2, _, cov_up_dp = self._twiss_terms(u, up, dp)
        sigma22 = self.cov(up, up) - cov_up_dp * cov_up_dp / cov_dp2
        return sigma22 / self.emittance(u, up, dp)

    def statistic(self, name, betagamma, p0, charge_e):
        """The Particles method ``name`` (particles/particles.py:311-390);
        betagamma and p0 of the bunch, charge_e the elementary charge."""
        if name.startswith('mean_'):
            return self.mean(name[5:])
        if name.startswith('sigma_'):
            return self.std(name[6:])
        if name in ('effective_normalized_emittance_z', 'epsn_z'):
            return 4 * np.pi * self.emittance('z', 'dp', None) * p0 / charge_e
        pl = name[-1]
        u, up = _U[pl]
        if name.startswith('effective_normalized_emittance_'):
            return self.emittance(u, up, None) * betagamma
        if name.startswith('epsn_'):
            return self.emittance(u, up, 'dp') * betagamma
        if name.startswith('dispersion_'):
            return self.dispersion(pl)
        if name.startswith('alpha_Twiss_'):
            return self.alpha(u, up, 'dp')
        if name.startswith('beta_Twiss_'):
            return self.beta(u, up, 'dp')
        if name.startswith('gamma_Twiss_'):
            return self.gamma(u, up, 'dp')
        raise KeyError(name)

