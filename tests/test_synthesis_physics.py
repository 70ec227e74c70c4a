"""The moment-tensor synthesis and the single-force weights give the
physical displacement (CPU, FP64 oracle columns, corrected layout).

Reciprocity: the displacement u_n at a surface receiver x_r from a moment
tensor M at the source point xi is M : grad u^(n)(xi), where u^(n) is the
field of a unit force along e_n at x_r.  That field comes from the library's
own single-force columns of the swapped problem (force at the surface,
receiver at the source depth), their orientation fixed by physics alone:
the free surface (sigma_rz = 0) makes the radial and vertical columns
opposite in orientation, the traction jump at the force (-F) gives its
direction, and a single-valued field at r -> 0 ties u_theta to u_r.  The
synthesis (grt_mt_weights, the combination grt_plan_synth applies) must
equal that displacement, Z up, R away from the source, T clockwise, for every
azimuthal family of the moment tensor."""
import math

import numpy as np
import pytest

from oracle import synth_oracle as SO

DISTS = np.array([15.0, 40.0])
ZS = 10.0005
UNITS = {"Mzz": [0, 0, 1, 0, 0, 0], "Mxx+Myy": [1, 1, 0, 0, 0, 0], "Mxx-Myy": [1, -1, 0, 0, 0, 0],
         "Mxy": [0, 0, 0, 1, 0, 0], "Mxz": [0, 0, 0, 0, 1, 0], "Myz": [0, 0, 0, 0, 0, 1]}


@pytest.fixture(scope="module")
def spectra(oracle):
    from grtm_cuda_gb300 import synth
    m, _ = synth.crust4_model()
    fix = oracle.FIX_ALL | oracle.STABLE | oracle.FIX_COLS | oracle.FIX_SHSRC

    def run(hs, hr, src):
        j = oracle.model(m["ztop"], m["vp"], m["vs"], m["rho"], m["qp"], m["qs"], hs, hr, src)
        oracle.setup(j, 0.1, 9, 0.0, 0.3, math.pi, oracle.K_FIXED, 2048, 0.0, fix)
        s, _ = oracle.run(j, DISTS, nthreads=0, want_sig=False)
        return s[:, : j.nw, :]

    return run(ZS, 0.0, 1), run(0.0, ZS, 0)     # moment tensor at depth, force at the surface


def _force_gradient(S, kind, th):
    """Gradient D[i][j] = d u_i / d x_j in (r, theta, z down) at the field point
    for a unit force at the origin: 'down', or horizontal with the field point
    at angle th from the force direction.  S: single-force spectra [nd, nw, 30]
    (0-4 displacement, 5-9 d/dz, 10-14 d/dr)."""
    r = DISTS[:, None]
    z = 0 * S[..., 0]
    c, s = math.cos(th), math.sin(th)
    if kind == "down":
        u, uz, ur, ut = ([S[..., 1], z, -S[..., 4]], [S[..., 6], z, -S[..., 9]], [S[..., 11], z, -S[..., 14]],
                         [z, z, z])
    else:
        u = [S[..., 0] * c, -S[..., 2] * s, -S[..., 3] * c]
        uz = [S[..., 5] * c, -S[..., 7] * s, -S[..., 8] * c]
        ur = [S[..., 10] * c, -S[..., 12] * s, -S[..., 13] * c]
        ut = [-S[..., 0] * s, -S[..., 2] * c, S[..., 3] * s]
    return [[ur[0], (ut[0] - u[1]) / r, uz[0]],
            [ur[1], (ut[1] + u[0]) / r, uz[1]],
            [ur[2], ut[2] / r, uz[2]]]


def _local(m6, psi):
    """Moment tensor (x north, y east, z down) in the basis (r-hat, theta-hat, z)
    at azimuth psi."""
    M = np.array([[m6[0], m6[3], m6[4]], [m6[3], m6[1], m6[5]], [m6[4], m6[5], m6[2]]])
    c, s = math.cos(psi), math.sin(psi)
    Q = np.array([[c, s, 0.0], [-s, c, 0.0], [0.0, 0.0, 1.0]])
    return Q @ M @ Q.T


def _reciprocal_zrt(S, m6, phi_deg):
    """Displacement (Z up, R away, T clockwise) at the receivers, by reciprocity."""
    phi = math.radians(phi_deg)
    psi = phi + math.pi               # the source seen from the receiver
    ML = _local(m6, psi)
    out = []
    for kind, th in (("down", 0.0), ("h", psi - phi), ("h", psi - phi - math.pi / 2)):
        D = _force_gradient(S, kind, th)
        out.append(sum(ML[i, j] * D[i][j] for i in range(3) for j in range(3)))
    out[0] = -out[0]                  # up
    return np.stack(out)


def test_library_weights_equal_the_restatement():
    import grtm_cuda_gb300 as g
    rng = np.random.default_rng(3)
    for _ in range(20):
        m6, phi = rng.normal(size=6), rng.uniform(0, 360)
        w = g.mt_weights(m6, phi)
        assert np.array_equal(w[:, 20:], np.zeros((3, 10)))
        assert np.allclose(w[:, :20], SO.weights(m6, phi), rtol=0, atol=1e-14)


@pytest.mark.parametrize("phi", [37.0, 200.0])
@pytest.mark.parametrize("name", list(UNITS))
def test_synthesis_equals_the_reciprocal_displacement(spectra, name, phi):
    import grtm_cuda_gb300 as g
    sT, sF = spectra
    m6 = np.array(UNITS[name], float)
    want = _reciprocal_zrt(sF, m6, phi)
    got = np.einsum("kc,dnc->kdn", g.mt_weights(m6, phi)[:, :20], sT[:, :, :20])
    for comp in range(3):
        scale = max(np.abs(want[comp]).max(), np.abs(got).max())
        assert np.abs(got[comp] - want[comp]).max() <= 1e-7 * scale, ("ZRT"[comp], name, phi)


def test_double_couple_and_explosion(spectra):
    import grtm_cuda_gb300 as g
    sT, sF = spectra
    for m6 in (g.dc_moment(30, 60, 90), g.dc_moment(123, 17, -45), np.array([1.0, 1, 1, 0, 0, 0])):
        for phi in (10.0, 130.0, 250.0):
            want = _reciprocal_zrt(sF, m6, phi)
            got = np.einsum("kc,dnc->kdn", g.mt_weights(m6, phi)[:, :20], sT[:, :, :20])
            assert np.abs(got - want).max() <= 1e-7 * np.abs(want).max()
    # an explosion has no transverse motion and no azimuthal dependence
    w = [g.mt_weights([1.0, 1, 1, 0, 0, 0], phi) for phi in (0.0, 77.0)]
    assert np.array_equal(w[0], w[1]) and not np.any(w[0][2])


@pytest.fixture(scope="module")
def force_spectra(oracle):
    from grtm_cuda_gb300 import synth
    m, _ = synth.crust4_model()
    fix = oracle.FIX_ALL | oracle.STABLE | oracle.FIX_COLS | oracle.FIX_SHSRC

    def run(hs, hr):
        j = oracle.model(m["ztop"], m["vp"], m["vs"], m["rho"], m["qp"], m["qs"], hs, hr, 0)
        oracle.setup(j, 0.1, 9, 0.0, 0.3, math.pi, oracle.K_FIXED, 2048, 0.0, fix)
        s, _ = oracle.run(j, DISTS, nthreads=0, want_sig=False)
        return s[:, : j.nw, :]

    return run(ZS, 0.0), run(0.0, ZS)       # force at depth / force at the surface (swapped)


@pytest.mark.parametrize("phi", [37.0, 200.0])
def test_single_force_weights_equal_the_reciprocal_displacement(force_spectra, phi):
    """grt_sf_weights: u_n(x_r) from a force F at xi equals F . u^(n)(xi), the
    field at the source point of a unit force along e_n at the receiver."""
    import grtm_cuda_gb300 as g
    s_src, s_rcv = force_spectra
    ph = math.radians(phi)
    psi = ph + math.pi
    Q = np.array([[math.cos(psi), math.sin(psi), 0.0], [-math.sin(psi), math.cos(psi), 0.0], [0.0, 0.0, 1.0]])
    for force in ([0.0, 0.0, 1.0], [1.0, 0.0, 0.0], [0.0, 1.0, 0.0], [0.3, -0.7, 0.5]):
        f = np.array(force)
        fl = Q @ f
        got = np.einsum("kc,dnc->kdn", g.sf_weights(f, phi), s_src[:, :, :15])
        want = []
        for kind, th in (("down", 0.0), ("h", psi - ph), ("h", psi - ph - math.pi / 2)):
            c, s = math.cos(th), math.sin(th)
            S = s_rcv
            u = ([S[..., 1], 0 * S[..., 1], -S[..., 4]] if kind == "down"
                 else [S[..., 0] * c, -S[..., 2] * s, -S[..., 3] * c])
            want.append(sum(fl[i] * u[i] for i in range(3)))
        want[0] = -want[0]                  # up
        want = np.stack(want)
        scale = np.abs(want).max()
        assert np.abs(got - want).max() <= 1e-12 * scale, (force, phi)
