"""Synchrotron.track on the GPU against the reference's own tracking of the
same machine (tests/golden/synchrotron/*.npz): smooth optics in three
segments with a linear longitudinal map in the middle, a damper after each
segment and a resonator wake; non-smooth optics with a two-harmonic
RFSystems at the end of the ring.  Plain FP64 form, coordinates within
1e-12 of their RMS."""
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip('torch')

GOLDEN = os.path.join(os.path.dirname(__file__), 'golden', 'synchrotron')
COORDS = ('x', 'xp', 'y', 'yp', 'z', 'dp')


@pytest.mark.parametrize('name', ['synchrotron_linear',
                                  'synchrotron_nonlinear'])
def test_synchrotron_tracking_matches_reference(name):
    from pyheadtail_gb300 import _native
    _native.load()
    from test_synchrotron_host import build, load
    from pyheadtail_gb300.particles.particles import Particles
    g = load(name)
    spec = json.loads(str(g['spec']))
    machine = build(spec)
    b = spec['bunch']
    coords = {k: g['init_' + k] for k in COORDS}
    bunch = Particles(b['n'], b['intensity'] / b['n'], machine.charge,
                      machine.mass, machine.circumference, machine.gamma,
                      coords_n_momenta_dict=coords)
    for _ in range(spec['n_turns']):
        machine.track(bunch)
    got = bunch.coords_numpy()
    for k in COORDS:
        r = g['final_' + k]
        err = np.max(np.abs(got[k] - r)) / np.sqrt(np.mean(r**2))
        assert err <= 1e-12, (name, k, err)
