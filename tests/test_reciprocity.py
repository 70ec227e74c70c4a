"""Source-receiver reciprocity of the FP64 oracle (CPU).

The reference's known-answer case pins a single force with a surface
receiver only.  Reciprocity pins the other branches of the recursion against
that one: swapping source and receiver depths exchanges the receiver-above-
source and receiver-below-source evaluations (green.cu:775-857 and 858-915),
which share no code beyond the layer terms.  Per (w, k), with the
coefficients of get_ypars_a_* (a0, a1, a2: radial and vertical P-SV parts of
orders m = 0, 1, 2; b1, b2: SH; the suffix t: the receiver-depth derivative):

* single force, G_ij(zr; zs) = G_ji(zs; zr): a0z, a1r and b1 are symmetric,
  a0r(zs, zr) = -a1z(zr, zs);
* moment tensor: its displacements are the source-coordinate derivatives of
  the single-force field, i.e. by reciprocity the single-force field of the
  swapped problem differentiated in its receiver depth (the t coefficients)
  or along the surface (a factor k) -- which ties get_src_tensor to
  get_src_single and the d/dz receiver terms.

All P-SV relations hold to rounding in the reference's formulas with the d/dz
quirks corrected; the SH ones need GRT_FIX_SHSRC (the reference's m = 1 and
m = 2 SH source terms share one reflection factor, green.cu:1409-1412)."""
import numpy as np
import pytest

TOPS = [0.0, 2.0, 10.0, 20.0, 35.0]
VP = [3.0, 5.8, 6.5, 7.0, 8.0]
VS = [v / 1.73 for v in VP]
RHO = [1.74 * v ** 0.25 for v in VP]
QP, QS = [200.0] * 5, [100.0] * 5

# index of each coefficient in the oracle's point output
A0R, A0Z, A1R, A1Z, A2R, A2Z, B1, B2 = range(8)
T = 8   # offset of the receiver-depth derivatives

# (zs, zr) pairs on the 4-layer crust (half-space top 35 km): receiver below /
# above the source in other layers, both in one layer (either order), the
# deepest layer over the half-space, surface and near-surface depths (the
# swapped problem puts the source at the receiver's depth, so neither lies in
# the half-space); other models take them scaled to their half-space depth
PAIRS = [(5.0, 15.0), (3.0, 12.0), (12.5, 27.0), (12.5, 14.0), (14.0, 12.5), (0.7, 1.9), (8.0, 34.0),
         (12.0, 0.0)]
POINTS = [(10, 0.05), (50, 0.3), (120, 1.1), (200, 2.2)]
TOL = 1e-9


def _coef(oracle, model, hs, hr, src, fix, iw, k):
    job = oracle.model(*model, hs, hr, src)
    oracle.setup(job, 0.1, 9, 0.0, 0.3, 2.0, oracle.K_REFERENCE, 0, fix=fix)
    return oracle.point(job, iw, k)


def _close(a, b):
    return abs(a - b) <= TOL * max(abs(a), abs(b), 1e-300)


def _models():
    from grtm_cuda_gb300 import synth
    m = synth.crust(np.random.default_rng(5), 12, 10.0)
    crust = (m["ztop"], m["vp"], m["vs"], m["rho"], m["qp"], m["qs"])
    return {"crust4": (TOPS, VP, VS, RHO, QP, QS), "crust12": crust}


def _pairs(model):
    scale = model[0][-1] / TOPS[-1]
    return [(zs * scale, zr * scale) for zs, zr in PAIRS]


@pytest.mark.parametrize("stable", [False, True])
@pytest.mark.parametrize("name", ["crust4", "crust12"])
def test_single_force_reciprocity(oracle, name, stable):
    model = _models()[name]
    fix = oracle.FIX_ALL | (oracle.STABLE if stable else 0)
    for zs, zr in _pairs(model):
        for iw, k in POINTS:
            a = _coef(oracle, model, zs, zr, 0, fix, iw, k)
            b = _coef(oracle, model, zr, zs, 0, fix, iw, k)
            for c in (A0Z, A1R, B1):
                assert _close(a[c], b[c]), (zs, zr, iw, k, c, a[c], b[c])
            assert _close(a[A0R], -b[A1Z]), (zs, zr, iw, k, a[A0R], b[A1Z])


def _tensor_relations(t, f, k):
    """Moment-tensor coefficients t of (zs -> zr) against the single-force
    coefficients f of (zr -> zs); returns (name, lhs, rhs) triples."""
    return [
        ("a0z", t[A0Z], f[T + A0Z]),
        ("a0r", t[A0R], -f[T + A1Z]),
        ("a1r", t[A1R], k * f[A1Z] - f[T + A1R]),
        ("a1z", t[A1Z], -k * f[A0Z] + f[T + A0R]),
        ("a2r", t[A2R], k * f[A1R]),
        ("a2z", t[A2Z], -k * f[A0R]),
        ("b1", t[B1], -f[T + B1]),
        ("b2", t[B2], k * f[B1]),
    ]


@pytest.mark.parametrize("atten_mu", [False, True])
@pytest.mark.parametrize("stable", [False, True])
@pytest.mark.parametrize("name", ["crust4", "crust12"])
def test_moment_tensor_reciprocity_with_sh_source_fix(oracle, name, stable, atten_mu):
    model = _models()[name]
    fix = oracle.FIX_ALL | oracle.FIX_SHSRC | (oracle.STABLE if stable else 0) | (oracle.ATTEN_MU if atten_mu else 0)
    for zs, zr in _pairs(model):
        for iw, k in POINTS:
            t = _coef(oracle, model, zs, zr, 1, fix, iw, k)
            f = _coef(oracle, model, zr, zs, 0, fix, iw, k)
            for nm, lhs, rhs in _tensor_relations(t, f, k):
                assert _close(lhs, rhs), (zs, zr, iw, k, nm, lhs, rhs)


def test_reference_sh_source_terms_break_reciprocity(oracle):
    """Without GRT_FIX_SHSRC the P-SV relations still hold, but the SH m = 1
    term fails wherever the receiver lies above the source (surface
    receivers) and the SH m = 2 term wherever it lies below."""
    model = _models()["crust4"]
    fix = oracle.FIX_ALL
    for zs, zr in PAIRS:
        above = zr < zs
        for iw, k in POINTS:
            t = _coef(oracle, model, zs, zr, 1, fix, iw, k)
            f = _coef(oracle, model, zr, zs, 0, fix, iw, k)
            rel = {nm: _close(lhs, rhs) for nm, lhs, rhs in _tensor_relations(t, f, k)}
            assert all(rel[nm] for nm in ("a0z", "a0r", "a1r", "a1z", "a2r", "a2z"))
            assert rel["b1"] != above and rel["b2"] == above, (zs, zr, iw, k, rel)


def test_sh_source_fix_changes_only_the_sh_coefficients(oracle):
    model = _models()["crust4"]
    for zs, zr in [(15.0, 4.0), (5.0, 15.0), (12.5, 14.0)]:
        for iw, k in POINTS:
            a = _coef(oracle, model, zs, zr, 1, oracle.FIX_ALL, iw, k)
            b = _coef(oracle, model, zs, zr, 1, oracle.FIX_ALL | oracle.FIX_SHSRC, iw, k)
            psv = [c for c in range(16) if c not in (B1, B2, T + B1, T + B2)]
            assert np.array_equal(a[psv], b[psv])
            sh_changed = b[B2] != a[B2] if zr > zs else b[B1] != a[B1]
            assert sh_changed
