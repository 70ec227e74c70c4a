"""Boundary conditions of the layered medium (CPU, FP64 oracle, per (w, k)):
the free surface is traction free, displacement and traction are continuous
across every internal interface, and at the source they jump by the source's
own discontinuity.

At a receiver on the surface, the receiver coefficients of every azimuthal
order m (a_m[0] radial, a_m[1] vertical, suffix t their receiver-depth
derivative; z down) must satisfy

  sigma_rz = 0:  a_m[0]_t = k a_m[1]
  sigma_zz = 0:  a_m[1]_t = -(1 - 2 beta^2 / alpha^2) k a_m[0]

with alpha, beta the top layer's attenuated velocities at that frequency
(the reference's attenuation law, green.cu:177-180).  The source terms,
the generalized reflection recursion, the free-surface reflection and the
receiver's d/dz terms all enter; no reference output does.  With the
reference's d/dz quirk F12 (this point's nu replaced by that of the list's
first point, green.cu:674-675) both conditions fail whenever the source lies
below the receiver's layer: the correction GRT_FIX_REXUT is the physical
one."""
import math

import numpy as np
import pytest

TOPS = [0.0, 2.0, 10.0, 20.0, 35.0]
VP = [3.0, 5.8, 6.5, 7.0, 8.0]
VS = [v / 1.73 for v in VP]
RHO = [1.74 * v ** 0.25 for v in VP]
QP, QS = [200.0] * 5, [100.0] * 5
T = 8
ORDERS = [(0, 1), (2, 3), (4, 5)]     # (radial, vertical) of m = 0, 1, 2
POINTS = [(1, 0.01), (10, 0.05), (50, 0.3), (120, 1.1), (200, 2.2)]
DT, LOG2N = 0.1, 9


def _models():
    from grtm_cuda_gb300 import synth
    m = synth.crust(np.random.default_rng(8), 15, 10.0)
    return {"crust4": (TOPS, VP, VS, RHO, QP, QS),
            "crust15": (m["ztop"], m["vp"], m["vs"], m["rho"], m["qp"], m["qs"])}


def _poisson_factor(model, w):
    """1 - 2 beta^2 / alpha^2 of the top layer at complex frequency w."""
    _, vp, vs, _, qp, qs = model
    lw = np.log(w / (2 * math.pi))
    a = vp[0] * (1 + lw / (math.pi * qp[0]) + 0.5j / qp[0])
    b = vs[0] * (1 + lw / (math.pi * qs[0]) + 0.5j / qs[0])
    return 1 - 2 * b * b / (a * a)


def _traction_residuals(oracle, model, hs, src, fix):
    """Worst relative residual of the shear and the normal condition."""
    job = oracle.model(*model, hs, 0.0, src)
    oracle.setup(job, DT, LOG2N, 0.0, 0.3, 2.0, oracle.K_REFERENCE, 0, fix=fix)
    shear = normal = 0.0
    for iw, k in POINTS:
        y = oracle.point(job, iw, k)
        c = _poisson_factor(model, complex(2 * math.pi * job.df * iw, -job.sigma))
        for r, z in ORDERS:
            if y[r] == 0 and y[z] == 0:
                continue           # single force has no m = 2 terms
            shear = max(shear, abs(y[T + r] - k * y[z]) / max(abs(y[T + r]), abs(k * y[z])))
            normal = max(normal, abs(y[T + z] + c * k * y[r]) / max(abs(y[T + z]), abs(c * k * y[r])))
    return shear, normal


@pytest.mark.parametrize("stable", [False, True])
@pytest.mark.parametrize("src", [0, 1])
@pytest.mark.parametrize("name", ["crust4", "crust15"])
def test_surface_receiver_traction_free(oracle, name, src, stable):
    model = _models()[name]
    fix = oracle.FIX_ALL | oracle.FIX_SHSRC | (oracle.STABLE if stable else 0)
    depth = model[0][-1]
    # source in the receiver's layer, and deeper ones
    for hs in (0.3 * model[0][1], 0.3 * depth, 0.7 * depth):
        shear, normal = _traction_residuals(oracle, model, hs, src, fix)
        assert shear <= 1e-12 and normal <= 1e-12, (hs, shear, normal)


def test_reference_dz_quirk_breaks_the_free_surface(oracle):
    model = _models()["crust4"]
    fix = oracle.STABLE | oracle.FIX_RLAYER        # F12 as in the reference
    for src in (0, 1):
        # the source in the receiver's layer: the quirk's slot is not used there
        shear, normal = _traction_residuals(oracle, model, 1.0, src, fix)
        assert shear <= 1e-12 and normal <= 1e-12
        # the source two layers down: both conditions fail
        shear, normal = _traction_residuals(oracle, model, 12.0, src, fix)
        assert shear > 0.1 and normal > 0.1, (shear, normal)


def _lame(model, i, w):
    """(lambda, mu) of layer i at complex frequency w as the method's stress
    rows have them: the real mu0 = rho beta0^2 of the layer table (green.cu:
    182, 2048) with the attenuated velocities alpha(w), beta(w) -- the medium
    of density rho (beta0 / beta(w))^2 -- so lambda = mu0 (alpha^2 / beta^2 - 2)."""
    _, vp, vs, rho, qp, qs = model
    lw = np.log(w / (2 * math.pi))
    a = vp[i] * (1 + lw / (math.pi * qp[i]) + 0.5j / qp[i])
    b = vs[i] * (1 + lw / (math.pi * qs[i]) + 0.5j / qs[i])
    mu = rho[i] * vs[i] ** 2
    return mu * (a * a / (b * b)) - 2 * mu, mu


def _lame_attenuated(model, i, w):
    """The standard viscoelastic pair, mu = rho beta(w)^2."""
    _, vp, vs, rho, qp, qs = model
    lw = np.log(w / (2 * math.pi))
    a = vp[i] * (1 + lw / (math.pi * qp[i]) + 0.5j / qp[i])
    b = vs[i] * (1 + lw / (math.pi * qs[i]) + 0.5j / qs[i])
    mu = rho[i] * b * b
    return rho[i] * a * a - 2 * mu, mu


def _jumps(oracle, model, hs, hr_lo, hr_hi, src, fix, lame_lo, lame_hi, iw, k):
    """Differences (below minus above) of (u_H, u_V, sigma_rz, sigma_zz) per
    order and of (v, mu v_z) per SH order between receivers at hr_lo < hr_hi."""
    ju = oracle.model(*model, hs, hr_lo, src)
    jl = oracle.model(*model, hs, hr_hi, src)
    for j in (ju, jl):
        oracle.setup(j, DT, LOG2N, 0.0, 0.3, 2.0, oracle.K_REFERENCE, 0, fix=fix)
    yu, yl = oracle.point(ju, iw, k), oracle.point(jl, iw, k)
    w = complex(2 * math.pi * ju.df * iw, -ju.sigma)
    (lu, mu_u), (ll, mu_l) = lame_lo(w), lame_hi(w)
    psv, sh = {}, {}
    for m, (r, z) in enumerate(ORDERS):
        if yu[r] == 0 and yu[z] == 0:
            continue
        up = (yu[r], yu[z], mu_u * (yu[T + r] - k * yu[z]), (lu + 2 * mu_u) * yu[T + z] + lu * k * yu[r])
        dn = (yl[r], yl[z], mu_l * (yl[T + r] - k * yl[z]), (ll + 2 * mu_l) * yl[T + z] + ll * k * yl[r])
        psv[m] = (up, dn)
    for m, b in ((1, 6), (2, 7)):
        if yu[b] != 0:
            sh[m] = ((yu[b], mu_u * yu[T + b]), (yl[b], mu_l * yl[T + b]))
    return psv, sh, w


def _rel(a, b):
    return abs(a - b) / max(abs(a), abs(b), 1e-300)


@pytest.mark.parametrize("src", [0, 1])
def test_continuity_across_interfaces(oracle, src):
    """Receivers 1e-10 km above and below each internal interface of a model
    whose Q changes from layer to layer (other layers, other propagators):
    displacement, sigma_rz, sigma_zz and the SH pair (v, mu v_z) agree across
    it; the residual shrinks in proportion to the gap."""
    model = _models()["crust15"]
    fix = oracle.FIX_ALL | oracle.FIX_SHSRC
    eps = 1e-10
    tops = model[0]
    for hs in (0.5 * tops[1], 0.5 * (tops[4] + tops[5]), 0.5 * (tops[-2] + tops[-1])):
        for i in (1, 2, 4, len(tops) - 2):
            for iw, k in POINTS:
                psv, sh, _ = _jumps(oracle, model, hs, tops[i] - eps, tops[i] + eps, src, fix,
                                    lambda w: _lame(model, i - 1, w), lambda w: _lame(model, i, w), iw, k)
                for up, dn in psv.values():
                    for a, b in zip(up, dn):
                        assert _rel(a, b) < 1e-7, (hs, i, iw, k)
                for up, dn in sh.values():
                    for a, b in zip(up, dn):
                        assert _rel(a, b) < 1e-7, (hs, i, iw, k)


def test_constitutive_law_is_the_unattenuated_mu(oracle):
    """The reference's stress rows take the real mu0 with attenuated velocities:
    tractions are continuous under that law and not under mu = rho beta(w)^2
    where Qs changes across an interface (a modelling convention kept as the
    reference has it)."""
    model = _models()["crust15"]
    fix = oracle.FIX_ALL | oracle.FIX_SHSRC
    eps, worst = 1e-10, 0.0
    i = 2
    zi = model[0][i]
    assert model[5][i - 1] != model[5][i]
    for iw, k in POINTS:
        psv, _, _ = _jumps(oracle, model, 0.3, zi - eps, zi + eps, 1, fix,
                           lambda w: _lame_attenuated(model, i - 1, w), lambda w: _lame_attenuated(model, i, w),
                           iw, k)
        for up, dn in psv.values():
            worst = max(worst, _rel(up[2], dn[2]), _rel(up[3], dn[3]))
    assert worst > 1e-3


@pytest.mark.parametrize("src", [0, 1])
def test_source_discontinuities(oracle, src):
    """Receivers 1e-10 km above and below the source: the field jumps by the
    source's own discontinuity, per unit force or moment, at every (w, k) --
    single force: [sigma_zz] = 1 (m = 0), [sigma_rz] = -1 and [mu v_z] = -1
    (m = 1), displacement continuous; moment tensor: [u_V] = -1/(lambda + 2 mu)
    and [sigma_rz] = -k lambda/(lambda + 2 mu) (m = 0), [u_H] = -1/mu (m = 1),
    [sigma_rz] = -k (m = 2), [v] = -1/mu (SH, m = 1), [mu v_z] = -k (SH, m = 2).
    The SH terms need GRT_FIX_SHSRC."""
    model = _models()["crust15"]
    fix = oracle.FIX_ALL | oracle.FIX_SHSRC
    eps = 1e-10
    tops = model[0]
    for hs in (0.5 * tops[1], 0.5 * (tops[6] + tops[7])):
        il = int(np.searchsorted(tops, hs)) - 1
        for iw, k in POINTS:
            psv, sh, w = _jumps(oracle, model, hs, hs - eps, hs + eps, src, fix,
                                lambda w: _lame(model, il, w), lambda w: _lame(model, il, w), iw, k)
            lam, mu = _lame(model, il, w)
            if src == 0:
                want = {0: (0, 0, 0, 1), 1: (0, 0, -1, 0)}
                want_sh = {1: (0, -1)}
            else:
                want = {0: (0, -1 / (lam + 2 * mu), -k * lam / (lam + 2 * mu), 0), 1: (-1 / mu, 0, 0, 0),
                        2: (0, 0, -k, 0)}
                want_sh = {1: (-1 / mu, 0), 2: (0, -k)}
            assert sorted(psv) == sorted(want) and sorted(sh) == sorted(want_sh)
            for m, (up, dn) in psv.items():
                scale = max(abs(x) for x in up + dn)
                for a, b, e in zip(up, dn, want[m]):
                    assert abs((b - a) - e) <= 1e-7 * scale, (hs, iw, k, m, b - a, e)
            for m, (up, dn) in sh.items():
                scale = max(abs(x) for x in up + dn)
                for a, b, e in zip(up, dn, want_sh[m]):
                    assert abs((b - a) - e) <= 1e-7 * scale, (hs, iw, k, m, b - a, e)


BRANCHES = {                     # (hs, hr) on the 4-layer crust
    "same layer, receiver below": (12.0, 14.0),
    "same layer, receiver above": (14.0, 12.0),
    "receiver above, other layer": (12.0, 3.0),
    "receiver below, other layer": (5.0, 15.0),
    "receiver in the half-space": (5.0, 40.0),
}


def _derivative_residual(oracle, hs, hr, fix, dz=1e-5):
    """Worst relative difference between the receiver-depth derivative
    coefficients (t) and central differences of the displacement coefficients
    in receiver depth, at fixed (w, k), both sources."""
    model = _models()["crust4"]
    worst = 0.0

    def coef(z, src, iw, k):
        j = oracle.model(*model, hs, z, src)
        oracle.setup(j, DT, LOG2N, 0.0, 0.3, 2.0, oracle.K_REFERENCE, 0, fix=fix)
        return oracle.point(j, iw, k)

    for src in (0, 1):
        for iw, k in POINTS[1:4]:
            y = coef(hr, src, iw, k)
            dy = (coef(hr + dz, src, iw, k) - coef(hr - dz, src, iw, k)) / (2 * dz)
            for c in range(8):
                scale = max(abs(dy[c]), abs(y[T + c]))
                if scale > 0:
                    worst = max(worst, abs(dy[c] - y[T + c]) / scale)
    return worst


@pytest.mark.parametrize("branch", list(BRANCHES))
def test_receiver_derivative_terms(oracle, branch):
    """The d/dz receiver terms are the receiver-depth derivatives of the
    displacement terms in every branch of the receiver propagation with the
    quirks corrected; the reference's d/dz quirks each break some branches:
    the doubled factor / reused product (GRT_FIX_DZ: green.cu:720, 842, 902)
    the receiver-above-source ones, the first point's nu (GRT_FIX_REXUT:
    green.cu:674-675) the others away from the source's own level."""
    hs, hr = BRANCHES[branch]
    assert _derivative_residual(oracle, hs, hr, oracle.FIX_ALL) <= 1e-7
    dz_quirk = _derivative_residual(oracle, hs, hr, oracle.FIX_RLAYER | oracle.FIX_REXUT)
    rexut_quirk = _derivative_residual(oracle, hs, hr, oracle.FIX_RLAYER | oracle.FIX_DZ)
    above = hr < hs
    assert (dz_quirk > 0.1) == above, dz_quirk
    expect_rexut = branch in ("same layer, receiver below", "receiver above, other layer",
                              "receiver below, other layer")
    assert (rexut_quirk > 0.1) == expect_rexut, rexut_quirk


@pytest.mark.parametrize("src", [0, 1])
def test_standard_viscoelastic_option_is_continuous(oracle, src):
    """With the oracle's ATTEN_MU (mu = rho beta(w)^2) the tractions are
    continuous under the standard law, where Q changes across interfaces."""
    model = _models()["crust15"]
    tops = model[0]
    fix = oracle.FIX_ALL | oracle.FIX_SHSRC | oracle.ATTEN_MU
    eps = 1e-10
    for i in (1, 2, 4):
        for iw, k in POINTS:
            psv, sh, _ = _jumps(oracle, model, 0.5 * (tops[5] + tops[6]), tops[i] - eps, tops[i] + eps, src, fix,
                                lambda w: _lame_attenuated(model, i - 1, w), lambda w: _lame_attenuated(model, i, w),
                                iw, k)
            for up, dn in list(psv.values()) + list(sh.values()):
                for a, b in zip(up, dn):
                    assert _rel(a, b) < 1e-7, (i, iw, k)
