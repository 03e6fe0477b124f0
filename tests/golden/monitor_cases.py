"""Monitor runs shared by the HDF5 layout fixture generator
(make_golden_monitors.py, which drives the reference's monitors) and the
host test of this repository's monitors: the constructor arguments and
the values every dump sees (bunch statistics, slice statistics,
coordinates), as functions of the step."""
import numpy as np

PARAMETERS = {'intensity': 2.5e11, 'n_turns_wake': 50, 'optics': 'smooth'}

BUNCH_STATS = ['mean_x', 'mean_xp', 'mean_y', 'mean_yp', 'mean_z', 'mean_dp',
               'sigma_x', 'sigma_y', 'sigma_z', 'sigma_dp', 'epsn_x',
               'epsn_y', 'epsn_z', 'macroparticlenumber']
SLICE_STATS = ['mean_x', 'mean_xp', 'mean_y', 'mean_yp', 'mean_z', 'mean_dp',
               'sigma_x', 'sigma_y', 'sigma_z', 'sigma_dp', 'epsn_x',
               'epsn_y', 'epsn_z', 'n_macroparticles_per_slice']
COORDS = ['x', 'xp', 'y', 'yp', 'z', 'dp', 'id']

# BunchMonitor: ten steps, a write every third, a four-step buffer (the
# last write is a partial one)
BUNCH_RUN = dict(n_steps=10, write_buffer_every=3, buffer_size=4)
# SliceMonitor: seven steps over five slices, a write every second step
SLICE_RUN = dict(n_steps=7, write_buffer_every=2, buffer_size=3, n_slices=5)
# ParticleMonitor: 11 macroparticles, every third stored, three dumps with
# one extra array
PARTICLE_RUN = dict(n=11, stride=3, n_dumps=3)


def bunch_value(stat, step):
    """Statistic ``stat`` of the bunch at ``step`` (float; an int for the
    macroparticle number)."""
    if stat == 'macroparticlenumber':
        return 1000 + 3 * step
    k = BUNCH_STATS.index(stat)
    return float(np.sin(1.3 * step + 0.7 * k) * 10.0**(-(k % 5) - 1))


def slice_value(stat, step, n_slices):
    """Per-slice statistic ``stat`` at ``step`` (n_slices values)."""
    if stat == 'n_macroparticles_per_slice':
        return (np.arange(n_slices, dtype=np.int32) * 7 + step) % 11
    k = SLICE_STATS.index(stat)
    i = np.arange(n_slices)
    return np.cos(0.9 * step + 0.4 * i + 0.3 * k) * 10.0**(-(k % 4) - 2)


def particle_arrays(step, n):
    """Coordinates (FP64) and ids (int32) of the bunch at dump ``step``,
    and the extra array passed to that dump."""
    i = np.arange(n)
    out = {q: np.sin(0.37 * i + 1.1 * step + j) * 10.0**(-j % 3 - 3)
           for j, q in enumerate(COORDS[:-1])}
    out['id'] = (i + 1).astype(np.int32)
    extra = {'kick_x': np.cos(0.5 * i - step) * 1e-6}
    return out, extra
