"""Boundary conditions of the layered medium (CPU, FP64 oracle, per (w, k)):
the free surface is traction free, and displacement and traction are
continuous across every internal interface.

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
    """Attenuated (lambda, mu) of layer i at complex frequency w."""
    _, vp, vs, rho, qp, qs = model
    lw = np.log(w / (2 * math.pi))
    a = vp[i] * (1 + lw / (math.pi * qp[i]) + 0.5j / qp[i])
    b = vs[i] * (1 + lw / (math.pi * qs[i]) + 0.5j / qs[i])
    mu = rho[i] * b * b
    return rho[i] * a * a - 2 * mu, mu


@pytest.mark.parametrize("src", [0, 1])
def test_continuity_across_interfaces(oracle, src):
    """Receivers 1e-10 km above and below each internal interface (other
    layers, other propagators): displacement, sigma_rz = mu (u_H,z - k u_V),
    sigma_zz = (lambda + 2 mu) u_V,z + lambda k u_H and the SH pair (v,
    mu v_z) agree across it; the residual shrinks in proportion to the gap."""
    model = _models()["crust4"]
    fix = oracle.FIX_ALL | oracle.FIX_SHSRC
    eps = 1e-10

    def rel(a, b):
        return abs(a - b) / max(abs(a), abs(b), 1e-300)

    for hs in (1.0, 12.0, 25.0):              # source above, between and below the interfaces
        for zi, (iu, il) in ((2.0, (0, 1)), (10.0, (1, 2)), (20.0, (2, 3))):
            ju = oracle.model(*model, hs, zi - eps, src)
            jl = oracle.model(*model, hs, zi + eps, src)
            for j in (ju, jl):
                oracle.setup(j, DT, LOG2N, 0.0, 0.3, 2.0, oracle.K_REFERENCE, 0, fix=fix)
            for iw, k in POINTS:
                yu, yl = oracle.point(ju, iw, k), oracle.point(jl, iw, k)
                w = complex(2 * math.pi * ju.df * iw, -ju.sigma)
                (lu, mu_u), (ll, mu_l) = _lame(model, iu, w), _lame(model, il, w)
                for r, z in ORDERS:
                    if yu[r] == 0 and yu[z] == 0:
                        continue
                    assert rel(yu[r], yl[r]) < 1e-7 and rel(yu[z], yl[z]) < 1e-7
                    assert rel(mu_u * (yu[T + r] - k * yu[z]), mu_l * (yl[T + r] - k * yl[z])) < 1e-7
                    assert rel((lu + 2 * mu_u) * yu[T + z] + lu * k * yu[r],
                               (ll + 2 * mu_l) * yl[T + z] + ll * k * yl[r]) < 1e-7
                for b in (6, 7):                    # SH: b1, b2
                    if yu[b] != 0:
                        assert rel(yu[b], yl[b]) < 1e-7
                        assert rel(mu_u * yu[T + b], mu_l * yl[T + b]) < 1e-7
