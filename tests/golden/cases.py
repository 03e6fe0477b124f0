"""Case specifications shared by the golden-fixture generator and the tests.

A case is a plain dict: beam parameters, an element list, the number of
turns and what to record.  ``make_golden.py`` builds the PyHEADTAIL
reference objects from it; ``oracle/cases.py`` builds the oracle objects;
the GPU tests build ``pyheadtail_gb300`` objects.  All three read the same
dict, so a fixture is only as trustworthy as the builders agreeing on it.

Sizes are small so that the committed fixtures stay around a megabyte.
"""
import numpy as np

C_SPS = 6911.5038378975451   # circumference used by the reference's tests
GAMMA = 27.7
Z_CUTS = (-0.69, 0.69)        # fixed +-3 sigma_z cuts for sigma_z = 0.23 m


def _alpha_c(Q_s=0.017, beta_z=230., gamma=GAMMA, C=C_SPS):
    # beta_z = |eta| C / (2 pi Q_s) with eta = alpha_c - gamma**-2 > 0
    return beta_z * 2 * np.pi * Q_s / C + gamma**-2


ALPHA_C = _alpha_c()


def beam_params(n, seed, **kw):
    p = dict(n=n, seed=seed, gamma=GAMMA, circumference=C_SPS,
             intensity=2.5e11, epsn_x=2.5e-6, epsn_y=2.5e-6, beta_x=50.,
             beta_y=50., alpha_x=0., alpha_y=0., sigma_z=0.23, sigma_dp=1e-3)
    p.update(kw)
    return p


def smooth_transverse(Q_x=20.13, Q_y=20.18, beta=50., chroma=None,
                      amplitude=None, n_segments=1, C=C_SPS):
    s = list(np.arange(0, n_segments + 1) * C / n_segments)
    m = n_segments + 1
    return dict(type='transverse', s=s, alpha_x=[0.] * m, beta_x=[beta] * m,
                D_x=[0.] * m, alpha_y=[0.] * m, beta_y=[beta] * m,
                D_y=[0.] * m, accQ_x=Q_x, accQ_y=Q_y, chroma=chroma,
                amplitude=amplitude)


def rf(h=(4620,), V=(4.5e6,), dphi=(0.,), alpha=ALPHA_C, p_increment=0.,
       D_x=0., D_y=0., shrink_transverse=True):
    return dict(type='rf', h=list(h), V=list(V), dphi=list(dphi),
                alpha=[alpha], p_increment=p_increment, D_x=D_x, D_y=D_y,
                shrink_transverse=shrink_transverse)


def linear_map(Q_s=0.017, alpha=ALPHA_C, D_x=0., D_y=0.):
    return dict(type='linear_map', Q_s=Q_s, alpha=[alpha], D_x=D_x, D_y=D_y)


def slicer(n_slices, z_cuts=Z_CUTS, n_sigma_z=None, mode='uniform_bin'):
    return dict(n_slices=n_slices,
                z_cuts=None if z_cuts is None else list(z_cuts),
                n_sigma_z=n_sigma_z, mode=mode)


def resonator(R=10e6, f=1e9, Q=1., n_turns_wake=1, kind='circular'):
    return dict(type='resonator', kind=kind, R=R, f=f, Q=Q,
                n_turns_wake=n_turns_wake)


def resistive_wall(b=0.02, L=C_SPS, sigma=5.8e7, dt_min=1e-12,
                   n_turns_wake=1, kind='circular'):
    return dict(type='resistive_wall', kind=kind, b=b, L=L, sigma=sigma,
                dt_min=dt_min, n_turns_wake=n_turns_wake)


TABLE_COLUMNS = ['time', 'constant_x', 'dipole_x', 'dipole_y', 'dipole_xy',
                 'dipole_yx', 'quadrupole_x', 'quadrupole_y', 'longitudinal']


def wake_table(file='wake_table_ultra.dat', columns=TABLE_COLUMNS,
               n_turns_wake=1):
    """A WakeTable source; ``file`` lives in this directory (synthetic
    tables written by make_wake_tables.py)."""
    return dict(type='wake_table', file=file, columns=list(columns),
                n_turns_wake=n_turns_wake)


def damper(dampingrate_x=50., dampingrate_y=50., phase=90, local_beta=None):
    """TransverseDamper (feedback/transverse_damper.py:15-94)."""
    return dict(type='damper', dampingrate_x=dampingrate_x,
                dampingrate_y=dampingrate_y, phase=phase,
                local_beta=local_beta)


def wake(sl, *sources):
    return dict(type='wake', slicer=sl, sources=list(sources))


def probe(sl, statistics=('mean_x', 'mean_y')):
    """Not an element of the reference: records a SliceSet of the beam in
    its current state (index, counts, statistics) without changing it."""
    return dict(type='probe', slicer=sl, statistics=list(statistics))


# every statistic of Particles (particles/particles.py:311-390); a case
# lists the ones recorded for the bunch after each recorded turn in
# record_bunch_stats
BUNCH_STATS = [
    'mean_x', 'mean_xp', 'mean_y', 'mean_yp', 'mean_z', 'mean_dp',
    'sigma_x', 'sigma_y', 'sigma_z', 'sigma_xp', 'sigma_yp', 'sigma_dp',
    'effective_normalized_emittance_x', 'effective_normalized_emittance_y',
    'effective_normalized_emittance_z', 'epsn_x', 'epsn_y', 'epsn_z',
    'dispersion_x', 'dispersion_y', 'alpha_Twiss_x', 'alpha_Twiss_y',
    'beta_Twiss_x', 'beta_Twiss_y', 'gamma_Twiss_x', 'gamma_Twiss_y']


# the C1 and C2 workloads at fixture size (full sizes are in bench.py)
CASES = {
    'transverse_linear': dict(
        beam=beam_params(1000, 11), n_turns=3,
        elements=[smooth_transverse()]),
    'transverse_chroma_amp': dict(
        beam=beam_params(1000, 12), n_turns=3,
        elements=[smooth_transverse(chroma=[5., 5.],
                                    amplitude=[1e-11, 1e-11, -5e-12])]),
    'transverse_segments_dispersion': dict(
        beam=beam_params(1000, 13), n_turns=3,
        elements=[dict(type='transverse', s=[0., 1000., 3500., C_SPS],
                       alpha_x=[0.3, -1.2, 0.7, 0.3],
                       beta_x=[50., 80., 20., 50.],
                       D_x=[2.0, 0.5, 1.1, 2.0],
                       alpha_y=[-0.4, 0.9, -0.2, -0.4],
                       beta_y=[40., 25., 70., 40.],
                       D_y=[0., 0.3, 0.0, 0.],
                       accQ_x=[0., 4.2, 13.6, 20.13],
                       accQ_y=[0., 6.1, 11.9, 20.18],
                       chroma=[[3., 120.], [-2., 40., 9000.]],
                       amplitude=[2e-11, -1e-11, 4e-12])]),
    'linear_map': dict(
        beam=beam_params(1000, 14), n_turns=3,
        elements=[linear_map()]),
    'rf_single': dict(
        beam=beam_params(1000, 15), n_turns=3, elements=[rf()]),
    'rf_double_harmonic': dict(
        beam=beam_params(1000, 16), n_turns=3,
        elements=[rf(h=(4620, 4 * 4620), V=(4.5e6, 0.45e6),
                     dphi=(0., np.pi))]),
    'rf_accelerating': dict(
        beam=beam_params(1000, 17), n_turns=3,
        elements=[smooth_transverse(), rf(p_increment=1e-21,
                                          D_x=0.7, D_y=0.)]),
    'slicer_fixed': dict(
        beam=beam_params(1000, 18), n_turns=1,
        elements=[probe(slicer(50), ['mean_x', 'mean_y', 'mean_z', 'mean_xp',
                                     'mean_yp', 'mean_dp', 'sigma_x',
                                     'sigma_z', 'epsn_x', 'eff_epsn_y',
                                     'epsn_z']),
                  probe(slicer(7, z_cuts=(-0.31, 0.05))),
                  probe(slicer(13, z_cuts=(0.2, -0.2))),
                  probe(slicer(20, z_cuts=None, n_sigma_z=3)),
                  probe(slicer(16, z_cuts=None))]),
    'wake_resonator': dict(
        beam=beam_params(1000, 19), n_turns=3,
        elements=[smooth_transverse(), linear_map(),
                  wake(slicer(50), resonator())]),
    'wake_multiturn': dict(
        beam=beam_params(1000, 20), n_turns=6,
        elements=[smooth_transverse(chroma=[2., 2.]), rf(),
                  wake(slicer(40), resonator(),
                       resistive_wall(n_turns_wake=4))]),
    'wake_dynamic_cuts': dict(
        beam=beam_params(1000, 21), n_turns=3,
        elements=[smooth_transverse(), rf(),
                  wake(slicer(30, z_cuts=None, n_sigma_z=4),
                       resonator(R=10.2e6, f=1.3e9),
                       resistive_wall(n_turns_wake=3))]),
    'wake_plates': dict(
        beam=beam_params(1000, 22), n_turns=3,
        elements=[smooth_transverse(), linear_map(),
                  wake(slicer(25), resonator(kind='parallel_horizontal'),
                       resonator(R=3e6, f=0.6e9, Q=0.5,
                                 kind='longitudinal'))]),
    # dispersion from the RF kick (D_x), dipolar, quadrupolar and
    # longitudinal wake kicks: every statistic of the bunch after the wake
    'bunch_statistics': dict(
        beam=beam_params(1500, 23, alpha_x=0.4, alpha_y=-0.3), n_turns=3,
        record_bunch_stats=BUNCH_STATS,
        elements=[smooth_transverse(chroma=[3., -2.]), rf(D_x=0.7, D_y=0.2),
                  wake(slicer(40), resonator(kind='parallel_horizontal'),
                       resonator(R=3e6, f=0.6e9, Q=0.5,
                                 kind='longitudinal'))]),
    # tabulated wakes: every kick kind (constant, dipolar, cross dipolar,
    # quadrupolar, longitudinal) from one table, multi-turn; and a
    # low-beta table
    'wake_table_multiturn': dict(
        beam=beam_params(1200, 24), n_turns=5,
        elements=[smooth_transverse(chroma=[1., 1.]), rf(),
                  wake(slicer(40), wake_table(n_turns_wake=3))]),
    'wake_table_lowbeta': dict(
        beam=beam_params(1200, 25), n_turns=3,
        elements=[smooth_transverse(), linear_map(),
                  wake(slicer(30), wake_table('wake_table_lowbeta.dat'))]),
    # the damper after a wake (its means see the kicks), a resistive one
    # in both planes and a reactive one in one plane before the maps
    'damper_resistive': dict(
        beam=beam_params(1200, 26), n_turns=4,
        elements=[smooth_transverse(chroma=[2., 2.]), rf(),
                  wake(slicer(40), resonator()), damper(20., 30.)]),
    'damper_reactive': dict(
        beam=beam_params(1200, 27), n_turns=4,
        elements=[damper(25., 0., phase=60., local_beta=50.),
                  smooth_transverse(), linear_map(),
                  wake(slicer(40), resonator())]),
    # UniformChargeSlicer: equal-count slices (Python's random module picks
    # the slices with one extra particle), the dot-product wake; fixed
    # cuts, and cuts from the bunch (n_sigma_z) with a resistive wall
    'charge_slicer': dict(
        beam=beam_params(1203, 28), n_turns=1, random_seed=5,
        elements=[probe(slicer(37, mode='uniform_charge'),
                        ['mean_x', 'mean_y', 'sigma_z', 'epsn_x']),
                  probe(slicer(16, z_cuts=(-0.2, 0.35),
                               mode='uniform_charge'))]),
    'wake_charge_slicer': dict(
        beam=beam_params(1200, 29), n_turns=4, random_seed=6,
        elements=[smooth_transverse(chroma=[-0.6, -0.6]), rf(),
                  wake(slicer(50, z_cuts=None, n_sigma_z=3,
                              mode='uniform_charge'),
                       resonator(),
                       resistive_wall(n_turns_wake=1))]),
    # the multi-turn wake workload (500 slices, resonator + 50-turn
    # resistive wall, RF) and the large-bunch physics (Q' 2, amplitude
    # detuning, 1000 slices, the same wakes) at fixture size
    'c3_full': dict(
        beam=beam_params(1000, 2), n_turns=8,
        elements=[smooth_transverse(), rf(),
                  wake(slicer(500), resonator(),
                       resistive_wall(n_turns_wake=50))]),
    'c5_full': dict(
        beam=beam_params(1000, 4), n_turns=5,
        elements=[smooth_transverse(chroma=[2., 2.],
                                    amplitude=[1e-11, 1e-11, -5e-12]),
                  rf(), wake(slicer(1000), resonator(),
                             resistive_wall(n_turns_wake=50))]),
    'c1_full': dict(
        beam=beam_params(1000, 0), n_turns=5,
        elements=[smooth_transverse(), linear_map(),
                  wake(slicer(50), resonator())]),
    'c2_full': dict(
        beam=beam_params(1000, 1), n_turns=5,
        elements=[smooth_transverse(chroma=[5., 5.],
                                    amplitude=[1e-11, 1e-11, -5e-12]),
                  rf(), wake(slicer(200), resonator())]),
}


# Synchrotron set-ups (machines/synchrotron.py): the machine's keyword
# arguments (charge / mass: e / m_p, added by the builders), the bunch and
# the extras of the turn loop.  Fixtures in synchrotron/<name>.npz.
P0_26GEV = 26e9 * 1.602176634e-19 / 299792458.0
SYNCHROTRON_CASES = {
    # smooth optics in three segments, RF parameters -> the linear map's
    # Q_s from the bucket formula, longitudinal map in the middle, a
    # damper after each segment and a resonator wake at the end
    'synchrotron_linear': dict(
        machine=dict(optics_mode='smooth', circumference=C_SPS, n_segments=3,
                     beta_x=54.6, beta_y=54.5, D_x=0.0, D_y=0.0,
                     accQ_x=20.13, accQ_y=20.18, Qp_x=2.0, Qp_y=-1.0,
                     app_x=3e-11, app_y=2e-11, app_xy=-1e-11,
                     longitudinal_mode='linear', alpha_mom_compaction=ALPHA_C,
                     h_RF=[4620], V_RF=[4.5e6], dphi_RF=[0.],
                     p_increment=0., p0=P0_26GEV, RF_at='middle'),
        bunch=dict(n=2000, seed=31, intensity=2.5e11, epsn_x=2e-6,
                   epsn_y=2e-6, sigma_z=0.23),
        damper_after_segments=(80., 120.),
        wake=dict(n_slices=40, R=10e6, f=1e9, Q=1.),
        n_turns=4),
    # non-smooth optics, two-harmonic RF at the end of the ring; the bunch
    # (cut at the separatrix by the reference) is handed over as data
    'synchrotron_nonlinear': dict(
        machine=dict(optics_mode='non-smooth',
                     s=[0., 2000., 4500., C_SPS],
                     alpha_x=[0.2, -0.8, 0.5, 0.2], beta_x=[50., 70., 30., 50.],
                     D_x=[0., 0., 0., 0.], alpha_y=[-0.3, 0.6, -0.1, -0.3],
                     beta_y=[45., 35., 60., 45.], D_y=[0., 0., 0., 0.],
                     accQ_x=[0., 6.3, 13.9, 20.13],
                     accQ_y=[0., 5.8, 12.7, 20.18], Qp_x=1.0, Qp_y=1.0,
                     longitudinal_mode='non-linear',
                     alpha_mom_compaction=ALPHA_C, h_RF=[4620, 4 * 4620],
                     V_RF=[4.5e6, 0.45e6], dphi_RF=[0., np.pi],
                     p_increment=0., p0=P0_26GEV, RF_at='end_of_transverse'),
        bunch=dict(n=2000, seed=32, intensity=2.5e11, epsn_x=2e-6,
                   epsn_y=2e-6, sigma_z=0.2),
        damper_after_segments=None, wake=None, n_turns=3),
}
