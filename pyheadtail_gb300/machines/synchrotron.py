"""Synchrotron: the one-turn map assembly (machines/synchrotron.py:15-647).

Builds the same ``one_turn_map`` as the reference -- the transverse
segments (smooth or non-smooth optics, chromaticity and amplitude detuning
shared over the segments) with the longitudinal map (``LinearMap`` or
``RFSystems``) inserted at the reference's position (``RF_at`` 'middle' or
'end_of_transverse') -- out of this package's elements, so that
``machine.track(bunch)`` and user loops over ``machine.one_turn_map`` run on
the GPU unchanged.

Set-up that needs the RF bucket's separatrix is not part of this package:
the Gaussian bunch of the 'non-linear' longitudinal mode (cut at the
separatrix), the bucket-matched bunch (``RF_bucket_distribution``) and the
z wrapper (``wrap_z``) raise NotImplementedError.  Such a bunch can be made
with PyHEADTAIL and handed over as coordinates
(``Particles(..., coords_n_momenta_dict=...)``).
"""
import numpy as np
from scipy.constants import c

from ..general.element import Element
from ..particles import generators
from ..trackers.detuners import AmplitudeDetuning, Chromaticity
from ..trackers.longitudinal_tracking import LinearMap, RFSystems
from ..trackers.transverse_tracking import TransverseMap


def bucket_Q_s(charge, mass, gamma, alpha0, harmonics, voltages):
    """RFBucket.Q_s (trackers/rf_bucket.py:268-279)."""
    beta = np.sqrt(1 - gamma**-2)
    p0 = np.sqrt(gamma**2 - 1) * mass * c
    eta0 = alpha0 - gamma**-2
    hV = sum([h * voltages[i] for i, h in enumerate(harmonics)])
    return np.sqrt(np.abs(charge) * np.abs(eta0) * hV /
                   (2 * np.pi * p0 * beta * c))


class Synchrotron(Element):
    """Same constructor as the reference (machines/synchrotron.py:16-246);
    see the module docstring for what is not built."""

    def __init__(self, optics_mode, charge=None, mass=None, p0=None,
                 circumference=None, n_segments=None, name=None, s=None,
                 alpha_x=None, beta_x=None, D_x=None, alpha_y=None,
                 beta_y=None, D_y=None, accQ_x=None, accQ_y=None, Qp_x=0,
                 Qp_y=0, app_x=0, app_y=0, app_xy=0, longitudinal_mode=None,
                 Q_s=None, alpha_mom_compaction=None, h_RF=None, V_RF=None,
                 dphi_RF=None, p_increment=None, RF_at='middle', wrap_z=False,
                 other_detuners=[], use_cython=False, *args, **kwargs):
        if use_cython:
            self.warns('Cython modules no longer in use. Using Python module '
                       'instead.\n')
        self.charge = charge
        self.mass = mass
        self.p0 = p0
        self.optics_mode = optics_mode
        self.longitudinal_mode = longitudinal_mode
        self.one_turn_map = []
        self._construct_transverse_map(
            optics_mode, circumference, n_segments, s, name, alpha_x, beta_x,
            D_x, alpha_y, beta_y, D_y, accQ_x, accQ_y, Qp_x, Qp_y, app_x,
            app_y, app_xy, other_detuners)
        self._construct_longitudinal_map(
            longitudinal_mode, np.atleast_1d(h_RF), np.atleast_1d(V_RF),
            np.atleast_1d(dphi_RF), alpha_mom_compaction, Q_s, p_increment,
            RF_at)
        if wrap_z:
            raise NotImplementedError('wrap_z: the z wrapper and buncher '
                                      '(synchrotron.py:613-647) are not part '
                                      'of this package')

    # -- the reference's scalar chain (synchrotron.py:247-281)
    @property
    def gamma(self):
        return self._gamma

    @gamma.setter
    def gamma(self, value):
        self._gamma = value
        self._beta = np.sqrt(1 - self.gamma**-2)
        self._betagamma = np.sqrt(self.gamma**2 - 1)
        self._p0 = self.betagamma * self.mass * c

    @property
    def beta(self):
        return self._beta

    @beta.setter
    def beta(self, value):
        self.gamma = 1.0 / np.sqrt(1 - value**2)

    @property
    def betagamma(self):
        return self._betagamma

    @betagamma.setter
    def betagamma(self, value):
        self.gamma = np.sqrt(value**2 + 1)

    @property
    def p0(self):
        return self._p0

    @p0.setter
    def p0(self, value):
        self.gamma = 1 / (c * self.mass) * np.sqrt(value**2 +
                                                   self.mass**2 * c**2)

    @property
    def Q_x(self):
        return np.atleast_1d(self.transverse_map.accQ_x)[-1]

    @property
    def Q_y(self):
        return np.atleast_1d(self.transverse_map.accQ_y)[-1]

    @property
    def Q_s(self):
        return np.atleast_1d(self.longitudinal_map.Q_s)[-1]

    def track(self, bunch, verbose=False):
        """synchrotron.py:294-298."""
        for m in self.one_turn_map:
            if verbose:
                self.prints('Tracking through:\n' + str(m))
            m.track(bunch)

    def install_after_each_transverse_segment(self, element_to_add):
        """synchrotron.py:300-307 (do not add elements that update the
        dispersion)."""
        new = []
        for element in self.one_turn_map:
            new.append(element)
            if any(element is m for m in self.transverse_map):
                new.append(element_to_add)
        self.one_turn_map = new

    # -- bunches
    def generate_6D_Gaussian_bunch(self, n_macroparticles, intensity, epsn_x,
                                   epsn_y, sigma_z, **kwargs):
        """synchrotron.py:309-360 for the 'linear' longitudinal mode:
        transversely matched, longitudinally matched to the linear focusing.
        ``kwargs`` go to Particles (e.g. precision='fp32')."""
        return self.gaussian_generator(n_macroparticles, intensity, epsn_x,
                                       epsn_y, sigma_z, **kwargs).generate()

    def gaussian_generator(self, n_macroparticles, intensity, epsn_x, epsn_y,
                           sigma_z, **kwargs):
        """The ParticleGenerator of generate_6D_Gaussian_bunch (its
        ``coordinates()`` are the host arrays of the bunch)."""
        if self.longitudinal_mode != 'linear':
            raise NotImplementedError(
                "a Gaussian bunch cut at the separatrix of a 'non-linear' "
                'bucket needs RFBucket, which is not part of this package')
        Q_s = self.longitudinal_map.Q_s
        eta = self.longitudinal_map.alpha_array[0] - self.gamma**-2
        beta_z = np.abs(eta) * self.circumference / 2.0 / np.pi / Q_s
        sigma_dp = sigma_z / beta_z
        epsx_geo = epsn_x / self.betagamma
        epsy_geo = epsn_y / self.betagamma
        opt = self.transverse_map.get_injection_optics()
        return generators.ParticleGenerator(
            macroparticlenumber=n_macroparticles, intensity=intensity,
            charge=self.charge, mass=self.mass,
            circumference=self.circumference, gamma=self.gamma,
            distribution_x=generators.gaussian2D(epsx_geo),
            alpha_x=opt['alpha_x'], beta_x=opt['beta_x'], D_x=opt['D_x'],
            distribution_y=generators.gaussian2D(epsy_geo),
            alpha_y=opt['alpha_y'], beta_y=opt['beta_y'], D_y=opt['D_y'],
            distribution_z=generators.gaussian2D_asymmetrical(
                sigma_u=sigma_z, sigma_up=sigma_dp),
            **kwargs)

    def generate_6D_Gaussian_bunch_matched(self, n_macroparticles, intensity,
                                           epsn_x, epsn_y, sigma_z=None,
                                           epsn_z=None, **kwargs):
        """synchrotron.py:362-410: the 'linear' mode's Gaussian bunch; the
        bucket-matched distribution of the 'non-linear' mode is not part
        of this package."""
        if self.longitudinal_mode == 'linear':
            assert sigma_z is not None
            return self.generate_6D_Gaussian_bunch(
                n_macroparticles, intensity, epsn_x, epsn_y, sigma_z,
                **kwargs)
        if self.longitudinal_mode == 'non-linear':
            raise NotImplementedError(
                'the RF-bucket matched distribution is host-side set-up of '
                'the reference; generate the bunch with PyHEADTAIL and pass '
                'its coordinates to Particles')
        raise ValueError('Unknown longitudinal mode!')

    # -- construction
    def _construct_transverse_map(self, optics_mode, circumference,
                                  n_segments, s, name, alpha_x, beta_x, D_x,
                                  alpha_y, beta_y, D_y, accQ_x, accQ_y, Qp_x,
                                  Qp_y, app_x, app_y, app_xy,
                                  other_detuners):
        """synchrotron.py:412-517."""
        if optics_mode == 'smooth':
            if circumference is None:
                raise ValueError('circumference has to be specified '
                                 'if optics_mode = "smooth"')
            if n_segments is None:
                raise ValueError('n_segments has to be specified '
                                 'if optics_mode = "smooth"')
            if s is not None:
                raise ValueError('s vector should not be provided '
                                 'if optics_mode = "smooth"')
            s = np.arange(0, n_segments + 1) * circumference / n_segments
            alpha_x = 0.0 * s
            beta_x = 0.0 * s + beta_x
            D_x = 0.0 * s + D_x
            alpha_y = 0.0 * s
            beta_y = 0.0 * s + beta_y
            D_y = 0.0 * s + D_y
        elif optics_mode == 'non-smooth':
            if circumference is not None:
                raise ValueError('circumference should not be provided '
                                 'if optics_mode = "non-smooth"')
            if n_segments is not None:
                raise ValueError('n_segments should not be provided '
                                 'if optics_mode = "non-smooth"')
            if s is None:
                raise ValueError('s has to be specified '
                                 'if optics_mode = "smooth"')
        else:
            raise ValueError('optics_mode not recognized')

        detuners = []
        if any(np.atleast_1d(Qp_x) != 0) or any(np.atleast_1d(Qp_y) != 0):
            detuners.append(Chromaticity(Qp_x, Qp_y))
        if app_x != 0 or app_y != 0 or app_xy != 0:
            detuners.append(AmplitudeDetuning(app_x, app_y, app_xy))
        detuners += other_detuners

        self.transverse_map = TransverseMap(
            s=s, alpha_x=alpha_x, beta_x=beta_x, D_x=D_x, alpha_y=alpha_y,
            beta_y=beta_y, D_y=D_y, accQ_x=accQ_x, accQ_y=accQ_y,
            detuners=detuners)
        self.circumference = s[-1]
        self.transverse_map.n_segments = len(s) - 1
        if name is None:
            self.transverse_map.name = ['P_%d' % ip for ip in range(len(s) - 1)]
            self.transverse_map.name.append('end_ring')
        else:
            self.transverse_map.name = name
        for i_seg, m in enumerate(self.transverse_map):
            m.i0, m.i1 = i_seg, i_seg + 1
            m.s0 = self.transverse_map.s[i_seg]
            m.s1 = self.transverse_map.s[i_seg + 1]
            m.name0 = self.transverse_map.name[i_seg]
            m.name1 = self.transverse_map.name[i_seg + 1]
            m.beta_x0 = self.transverse_map.beta_x[i_seg]
            m.beta_x1 = self.transverse_map.beta_x[i_seg + 1]
            m.beta_y0 = self.transverse_map.beta_y[i_seg]
            m.beta_y1 = self.transverse_map.beta_y[i_seg + 1]
        for m in self.transverse_map:
            self.one_turn_map.append(m)

    def _construct_longitudinal_map(self, longitudinal_mode, h_RF, V_RF,
                                    dphi_RF, alpha_mom_compaction, Q_s,
                                    p_increment, RF_at):
        """synchrotron.py:519-611."""
        if longitudinal_mode is None:
            return
        have_rf = (h_RF[0] is not None and V_RF[0] is not None and
                   dphi_RF[0] is not None and alpha_mom_compaction is not None
                   and p_increment is not None)
        if RF_at == 'middle':
            for insert_before, si in enumerate(self.transverse_map.s):
                if si > 0.5 * self.circumference:
                    break
            insert_before -= 1
        elif RF_at == 'end_of_transverse':
            insert_before = -1
        else:
            raise ValueError('RF_at=%s not recognized!')

        if longitudinal_mode == 'linear':
            if V_RF[0] is not None and Q_s is not None:
                raise ValueError('Q_s and V_RF cannot be provided at the '
                                 'same time')
            if Q_s is None:
                if not have_rf:
                    raise AttributeError('Q_s not available!')
                Q_s = bucket_Q_s(self.charge, self.mass, self.gamma,
                                 np.atleast_1d(alpha_mom_compaction)[0],
                                 h_RF, V_RF)
            self.longitudinal_map = LinearMap(
                np.atleast_1d(alpha_mom_compaction), self.circumference, Q_s,
                D_x=self.transverse_map.D_x[insert_before],
                D_y=self.transverse_map.D_y[insert_before])
        elif longitudinal_mode == 'non-linear':
            if Q_s is not None:
                raise ValueError('Q_s cannot be provided if longitudinal '
                                 'mode is non-linear')
            self.longitudinal_map = RFSystems(
                charge=self.charge, mass=self.mass,
                circumference=self.circumference,
                gamma_reference=self.gamma,
                voltage_list=np.atleast_1d(V_RF),
                harmonic_list=np.atleast_1d(h_RF),
                phi_offset_list=np.atleast_1d(dphi_RF),
                alpha_array=np.atleast_1d(alpha_mom_compaction),
                p_increment=p_increment,
                D_x=self.transverse_map.D_x[insert_before],
                D_y=self.transverse_map.D_y[insert_before])
        else:
            raise NotImplementedError('Something wrong with longitudinal_mode')

        if insert_before == -1:
            self.one_turn_map.append(self.longitudinal_map)
        else:
            self.one_turn_map.insert(insert_before, self.longitudinal_map)


class BasicSynchrotron(Synchrotron):
    """Deprecated alias of Synchrotron (synchrotron.py:675-687)."""

    def __init__(self, *args, **kwargs):
        self.warns('"BasicSynchrotron" will be removed in the near future. '
                   'Use "Synchrotron" instead.\n')
        super(BasicSynchrotron, self).__init__(*args, **kwargs)
