"""Write the synthetic wake tables used by the WakeTable cases.

    python tests/golden/make_wake_tables.py

The tables follow the column conventions of PyHEADTAIL's WakeTable
(impedances/wakes.py:167-212): time in ns, transverse components in
V/pC/mm, longitudinal in V/pC, one row per time sample.  The values are
made up here from damped resonator shapes and a 1/sqrt(t) tail (no
measured machine data):

* wake_table_ultra.dat: time from 0 (the ultrarelativistic branch: every
  transverse component is 0 at t = 0), dense to 20 ns, then geometric to
  60 us so that multi-turn wakes of the SPS-like test ring (23 us per turn)
  stay inside the table;
* wake_table_lowbeta.dat: time from -5 ns (the low-beta branch), to 10 ns.
"""
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))

COLUMNS = ['time', 'constant_x', 'dipole_x', 'dipole_y', 'dipole_xy',
           'dipole_yx', 'quadrupole_x', 'quadrupole_y', 'longitudinal']


def shapes(t_ns):
    """Made-up wake components at times t_ns (ns)."""
    t = np.asarray(t_ns, dtype=np.float64)
    tp = np.clip(t, 0, None)
    res = lambda a, f, d: a * np.exp(-tp / d) * np.sin(2 * np.pi * f * tp)
    tail = lambda a: a * (1 - np.exp(-tp / 0.3)) / np.sqrt(1 + tp)
    cols = [
        0.02 * res(1., 0.4, 3.) + 0.01 * tail(1.),          # constant_x
        res(35., 1.0, 1.5) + tail(4.),                       # dipole_x
        res(28., 1.3, 1.2) + tail(3.),                       # dipole_y
        res(3., 0.7, 2.0),                                   # dipole_xy
        res(2., 0.9, 2.5),                                   # dipole_yx
        res(-12., 1.0, 1.5) - tail(1.),                      # quadrupole_x
        res(10., 1.3, 1.2) + tail(1.),                       # quadrupole_y
        8. * np.exp(-tp / 0.8) * np.cos(2 * np.pi * 0.6 * tp),   # longitudinal
    ]
    # below t = 0 (low-beta tables) every component is non-zero, rising
    # towards t = 0
    pre = np.where(t < 0, np.exp(np.minimum(t, 0.) / 0.7), 0.)
    out = [c + 0.3 * (k + 1) * pre for k, c in enumerate(cols)]
    return np.column_stack([t] + out)


def main():
    t_dense = np.linspace(0., 20., 401)
    t_far = np.geomspace(20., 6e4, 150)[1:]
    ultra = shapes(np.concatenate([t_dense, t_far]))
    low = shapes(np.linspace(-5., 10., 301))
    fmt = '%.12e'
    np.savetxt(os.path.join(HERE, 'wake_table_ultra.dat'), ultra, fmt=fmt,
               delimiter='\t')
    np.savetxt(os.path.join(HERE, 'wake_table_lowbeta.dat'), low, fmt=fmt,
               delimiter='\t')


if __name__ == '__main__':
    main()
