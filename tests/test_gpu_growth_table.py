"""Growth rate with a tabulated wake and a transverse damper, as the
reference's table-wake simulation test (tests/simulation_tests/
test_wake_table.py:86-120) measures it, on this repository's synthetic
table (dipolar columns, 3-turn memory), a resistive damper (3000 turns),
RF h=4620 and 2e4 macroparticles at 1.6e11 over 2000 turns: the
horizontal plane is unstable, the vertical one is damped.

The centroids come from Particles.mean_x / mean_y (one statistics pass per
turn, with the wake kicks still pending).  Bars against the FP64 oracle:
FP64 within 1e-6 relative, FP32 (tensor-core wake) within 2 %."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip('torch')

N_TURNS = 2000
COLUMNS = ['time', 'off_cx', 'dipole_x', 'dipole_y', 'off_dxy', 'off_dyx',
           'off_qx', 'off_qy', 'off_l']   # only the dipolar columns act


def _spec():
    import cases as C
    return dict(beam=C.beam_params(20000, 3, intensity=1.6e11),
                n_turns=N_TURNS, elements=[
                    C.smooth_transverse(), C.rf(),
                    C.wake(C.slicer(100),
                           C.wake_table(columns=COLUMNS, n_turns_wake=3)),
                    C.damper(3000., 3000.)])


def _run(make_elements, beam):
    els = [el for _, el in make_elements(_spec(), beam)]
    cx = np.zeros(N_TURNS)
    cy = np.zeros(N_TURNS)
    for t in range(N_TURNS):
        for el in els:
            el.track(beam)
        cx[t], cy[t] = beam.mean_x(), beam.mean_y()
    return cx, cy


def test_table_wake_with_damper_growth_rate():
    import gpu_cases as G
    from oracle import cases as OC
    from test_gpu_growth import growth_rate
    spec = _spec()
    ob = OC.make_beam(spec['beam'])
    coords = ob.coords()
    ox, oy = _run(OC.make_elements, ob)
    g_ref = (growth_rate(ox), growth_rate(oy))
    assert g_ref[0] > 5e-4 and g_ref[1] < 0, g_ref   # x unstable, y damped
    for precision, tol in (('fp64', 1e-6), ('fp32', 2e-2)):
        beam = G.make_beam(spec['beam'], coords, precision=precision)
        gx = growth_rate(_run(G.make_elements, beam)[0])
        rel = abs(gx - g_ref[0]) / g_ref[0]
        print('table wake + damper growth %s: %.6e vs oracle %.6e (rel %.2e)'
              % (precision, gx, g_ref[0], rel))
        assert rel <= tol, (precision, gx, g_ref)
