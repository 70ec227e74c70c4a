"""Seismogram synthesis restated in numpy -- TEST INFRASTRUCTURE ONLY.

Only tests/ may import this module.  The reference stops at the Green's
function columns (cusrc/popm/func/green.cu:1650-1691, moment-tensor columns
0-9 displacement); this restates the library's documented combination of
those columns for a moment tensor and azimuth, and the source-time
convolution at the complex frequency (a damped circular convolution), so the
fused GPU kernel can be checked against it on the same columns.
"""
import numpy as np


def dc_moment(strike, dip, rake, m0=1.0):
    """Aki & Richards, Box 4.4 (x north, y east, z down): (Mxx, Myy, Mzz, Mxy, Mxz, Myz)."""
    f, d, l = np.radians([strike, dip, rake])
    mxx = -m0 * (np.sin(d) * np.cos(l) * np.sin(2 * f) + np.sin(2 * d) * np.sin(l) * np.sin(f) ** 2)
    myy = m0 * (np.sin(d) * np.cos(l) * np.sin(2 * f) - np.sin(2 * d) * np.sin(l) * np.cos(f) ** 2)
    mzz = m0 * np.sin(2 * d) * np.sin(l)
    mxy = m0 * (np.sin(d) * np.cos(l) * np.cos(2 * f) + 0.5 * np.sin(2 * d) * np.sin(l) * np.sin(2 * f))
    mxz = -m0 * (np.cos(d) * np.cos(l) * np.cos(f) + np.cos(2 * d) * np.sin(l) * np.sin(f))
    myz = -m0 * (np.cos(d) * np.cos(l) * np.sin(f) - np.cos(2 * d) * np.sin(l) * np.cos(f))
    return np.array([mxx, myy, mzz, mxy, mxz, myz])


def weights(m, phi_deg):
    """[3 (Z, R, T), 20] weights of the moment-tensor columns at azimuth phi
    (the receiver's azimuth from the source, clockwise from north) for
    displacement Z up, R away from the source, T clockwise.  Relative to the
    column families the horizontal-isotropic term (columns 2, 9) and the
    m = 1 terms (1, 5, 7) enter with a minus sign: the m = 0 and m = 2 parts of
    the horizontal moments share the coefficients a2 with u_z = a2z k (h J0 -
    c2 J2), and the m = 1 columns carry the opposite orientation -- the
    signs for which every family equals the displacement reciprocity gives."""
    ph = np.radians(phi_deg)
    w2c, w2s, w1c, w1s = 0.5 * (m[0] - m[1]), m[3], -m[4], -m[5]
    w0, w0h = m[2], -0.5 * (m[0] + m[1])
    c2 = w2c * np.cos(2 * ph) + w2s * np.sin(2 * ph)
    s2 = -w2c * np.sin(2 * ph) + w2s * np.cos(2 * ph)
    c1 = w1c * np.cos(ph) + w1s * np.sin(ph)
    s1 = -w1c * np.sin(ph) + w1s * np.cos(ph)
    w = np.zeros((3, 20))
    w[0, 6], w[0, 7], w[0, 8], w[0, 9] = c2, c1, w0, w0h
    w[1, 0], w[1, 1], w[1, 3], w[1, 2] = c2, c1, w0, w0h
    w[2, 4], w[2, 5] = s2, s1
    return w


def synth(traces, m, azimuth, dt, sigma, t0=0.0, stf=None):
    """traces [nd, 20, N] -> seismograms [nd, 3, N]: combination, then
    dt sum_m s_m G(t - m dt) as the damped circular convolution the
    complex-frequency method implies."""
    nd, _, N = traces.shape
    az = np.broadcast_to(np.asarray(azimuth, np.float64), (nd,))
    out = np.einsum("dkc,dcn->dkn", np.stack([weights(m, a) for a in az]), traces)
    if stf is None:
        return out
    t = np.arange(N) * dt
    damp = np.exp(sigma * (t + t0))
    s = np.zeros(N)
    s[:len(stf)] = stf
    z = dt * s * np.exp(-sigma * t)
    g = out / damp
    conv = np.real(np.fft.ifft(np.fft.fft(g, axis=-1) * np.fft.fft(z), axis=-1))
    return conv * damp
