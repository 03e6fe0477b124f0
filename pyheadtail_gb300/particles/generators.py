"""Seeded bunch generation for the GPU Particles.

Restates the part of PyHEADTAIL's particles/generators.py that the turn-loop
workloads use: ``gaussian2D`` (:428-443), ``gaussian2D_asymmetrical``
(:446-459), the linear transverse matcher (:106-153) and
``ParticleGenerator`` (:299-405, draw order x, xp, y, yp, z, dp of
``_create_phase_space`` :377-395).  The draws use NumPy's global legacy RNG
exactly as the reference does, so ``np.random.seed(s)`` followed by
``generate()`` yields the reference's bunch bit for bit; the coordinates are
then copied to the GPU in the requested precision.
"""
import numpy as np

from .particles import Particles


def gaussian2D(emittance_geo):
    def _gaussian2D(n_particles):
        std = np.sqrt(emittance_geo)
        return [np.random.normal(loc=0., scale=std, size=n_particles),
                np.random.normal(loc=0., scale=std, size=n_particles)]
    return _gaussian2D


def gaussian2D_asymmetrical(sigma_u, sigma_up):
    def _gaussian2D(n_particles):
        return [np.random.normal(loc=0., scale=sigma_u, size=n_particles),
                np.random.normal(loc=0., scale=sigma_up, size=n_particles)]
    return _gaussian2D


def transverse_linear_matcher(alpha, beta, dispersion=None):
    M00 = np.sqrt(beta)
    M01 = 0
    M10 = -alpha / np.sqrt(beta)
    M11 = np.sqrt(1. / beta)

    def _match(coords, direction):
        u = coords[direction[0]]
        uc = u.copy()
        up = coords[direction[1]]
        u = M00 * u + M01 * up
        up = M10 * uc + M11 * up
        if dispersion:
            u += dispersion * coords['dp']
        coords[direction[0]] = u
        coords[direction[1]] = up
    return _match


class ParticleGenerator(object):
    """Generate a GPU Particles from per-plane distributions (transverse
    planes linearly matched to alpha / beta)."""

    def __init__(self, macroparticlenumber, intensity, charge, mass,
                 circumference, gamma, distribution_x=None, alpha_x=0.,
                 beta_x=1., D_x=None, distribution_y=None, alpha_y=0.,
                 beta_y=1., D_y=None, distribution_z=None, Qs=None, eta=None,
                 *args, **kwargs):
        self.macroparticlenumber = macroparticlenumber
        self.intensity = intensity
        self.charge, self.mass = charge, mass
        self.circumference, self.gamma = circumference, gamma
        self.distribution_x = distribution_x
        self.distribution_y = distribution_y
        self.distribution_z = distribution_z
        self.linear_matcher_z = None
        if Qs is not None and eta is not None:
            beta_z = np.abs(eta) * circumference / (2. * np.pi * Qs)
            self.linear_matcher_z = transverse_linear_matcher(0., beta_z)
        self.linear_matcher_x = transverse_linear_matcher(alpha_x, beta_x, D_x)
        self.linear_matcher_y = transverse_linear_matcher(alpha_y, beta_y, D_y)
        self.kwargs = kwargs

    def coordinates(self):
        """The matched coordinates as float64 NumPy arrays (host)."""
        n = self.macroparticlenumber
        coords = {}
        if self.distribution_x is not None:
            u = self.distribution_x(n)
            coords['x'], coords['xp'] = np.ascontiguousarray(u[0]), \
                np.ascontiguousarray(u[1])
        if self.distribution_y is not None:
            u = self.distribution_y(n)
            coords['y'], coords['yp'] = np.ascontiguousarray(u[0]), \
                np.ascontiguousarray(u[1])
        if self.distribution_z is not None:
            u = self.distribution_z(n)
            coords['z'], coords['dp'] = np.ascontiguousarray(u[0]), \
                np.ascontiguousarray(u[1])
        if self.linear_matcher_z is not None:
            self.linear_matcher_z(coords, ['z', 'dp'])
        if self.distribution_x is not None:
            self.linear_matcher_x(coords, ['x', 'xp'])
        if self.distribution_y is not None:
            self.linear_matcher_y(coords, ['y', 'yp'])
        return coords

    def generate(self):
        coords = self.coordinates()
        return Particles(self.macroparticlenumber,
                         self.intensity / self.macroparticlenumber,
                         self.charge, self.mass, self.circumference,
                         self.gamma, coords_n_momenta_dict=coords,
                         **self.kwargs)


def gaussian_bunch_coordinates(n, seed, gamma, epsn_x, epsn_y, beta_x, beta_y,
                               sigma_z, sigma_dp, alpha_x=0., alpha_y=0.):
    """The seeded 6D Gaussian of the turn-loop workloads (host float64)."""
    betagamma = np.sqrt(gamma**2 - 1)
    np.random.seed(seed)
    g = ParticleGenerator(n, 1., 1., 1., 1., gamma,
                          gaussian2D(epsn_x / betagamma), alpha_x, beta_x,
                          None, gaussian2D(epsn_y / betagamma), alpha_y,
                          beta_y, None,
                          gaussian2D_asymmetrical(sigma_z, sigma_dp))
    return g.coordinates()
