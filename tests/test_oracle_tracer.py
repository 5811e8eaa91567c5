"""Oracle checks of the tracer extensions (CPU): the upwind-biased flux and
the frozen flow keep the flux form's conservation, and a uniform tracer is
advected identically by both face rules."""
import numpy as np
import pytest

from oracle import OracleBackend
from swm_gb300.host import synthetic
from swm_gb300.host.driver import Driver


def _run(case, nsteps):
    o = OracleBackend(tracer_nan_guard=True)
    d = Driver(case, o)
    d.init(with_diag=False)
    d.run(nsteps, with_diag=False)
    return o


def _mass(o, t):
    cos = o.lat('cos_eta')
    return float((o.tracer_field(t, 'CH0') * cos[:, None]).sum())


@pytest.mark.parametrize('flux', [0, 1])
def test_tracer_mass_conserved_without_relaxation(flux):
    case = synthetic.tracer_flow(40, nsteps=60, flux=flux)
    for t in case['tracers']:
        t['gamma_c'] = 0.0
    o0 = _run(case, 0)
    m0 = [_mass(o0, t) for t in range(2)]
    o = _run(case, 60)
    for t in range(2):
        assert abs(_mass(o, t) - m0[t]) <= 1e-12 * abs(m0[t]), t
        assert np.isfinite(o.tracer_field(t, 'CH0')).all()


def test_frozen_flow_keeps_the_state():
    case = synthetic.tracer_flow(32, nsteps=20)
    o = _run(case, 20)
    np.testing.assert_array_equal(o.field('u'), case['ic']['u'] * o.ocean('u'))
    np.testing.assert_array_equal(o.field('v'), case['ic']['v'] * o.ocean('v'))


def test_uniform_tracer_same_under_both_face_rules():
    res = []
    for flux in (0, 1):
        case = synthetic.tracer_flow(32, nsteps=30, flux=flux, n_tracers=1)
        c = np.full(case['H'].shape, 0.3)
        case['tracers'][0].update(field_C=c, field_C0=c.copy(), gamma_c=0.0)
        res.append(_run(case, 30).tracer_field(0, 'CH0'))
    np.testing.assert_allclose(res[0], res[1], rtol=1e-13, atol=1e-13)


def test_upwind_biased_differs_from_centred_on_a_front():
    out = []
    for flux in (0, 1):
        case = synthetic.tracer_flow(40, nsteps=40, flux=flux, n_tracers=1)
        c = (np.arange(case['H'].shape[1])[None, :] > 20) * np.ones(case['H'].shape)
        case['tracers'][0].update(field_C=c, field_C0=c.copy(), gamma_c=0.0, kappa_h=0.0)
        o = _run(case, 40)
        out.append(o.tracer_field(0, 'CH0') / 100.0)
    assert np.abs(out[0] - out[1]).max() > 1e-6
