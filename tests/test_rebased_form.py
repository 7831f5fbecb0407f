"""The algebra of the rebased FP32 form (precision FP32_RB), in float64 on the
CPU.  The GPU kernels run the PT iteration on the change since an FP64 base:
H = H_b + delta, w = w_b + omega, with
  omega <- omega - c (t_b + omega + u_delta),   t_b = w_b + u(H_b),
  delta <- delta - e (R_b + delta/dt + sum_d (omega_R - omega_L) sigma_d),
  R_b = (H_b - Hold)/dt + sum_d (w_b,R - w_b,L) sigma_d,
and for D = H^3 (faces: s = H_L + H_R, g = H_R - H_L, u = s^3 g)
  u_delta = u(H_b + delta) - u(H_b) = s_d (3 s (s + s_d) + s_d^2) g + (s + s_d)^3 g_d.
These tests check that one such iteration equals one plain iteration
  w <- w - c (w + u(H)),   H <- H - e ((H - Hold)/dt + sum_d (w_R - w_L) sigma_d)
on the summed state, so the form changes only where rounding happens.  The
last test checks the defect-correction form's linearised flux (FP32_DC)
against the same flux change."""
import numpy as np


def faces(H, axis):
    L = np.take(H, np.arange(H.shape[axis] - 1), axis=axis)
    R = np.take(H, np.arange(1, H.shape[axis]), axis=axis)
    return L, R


def u_nonlin(H, axis):
    L, R = faces(H, axis)
    s, g = L + R, R - L
    return s ** 3 * g


def u_delta(Hb, d, axis):
    L, R = faces(Hb, axis)
    dL, dR = faces(d, axis)
    s, g = L + R, R - L
    sd, gd = dL + dR, dR - dL
    return sd * (3 * s * (s + sd) + sd ** 2) * g + (s + sd) ** 3 * gd


def div(w, axis, shape):
    """sum over faces of w_R - w_L at the inner cells, one axis."""
    out = np.zeros(shape)
    sl_in = [slice(1, -1)] * len(shape)
    dw = np.diff(w, axis=axis)
    sl_w = [slice(1, -1)] * len(shape)
    sl_w[axis] = slice(None)
    out[tuple(sl_in)] = dw[tuple(sl_w)]
    return out


def test_flux_change_identity():
    rng = np.random.default_rng(1)
    Hb = 1.0 + rng.random((9, 7))
    d = 1e-3 * rng.standard_normal((9, 7))
    for axis in (0, 1):
        exact = u_nonlin(Hb + d, axis) - u_nonlin(Hb, axis)
        assert np.allclose(u_delta(Hb, d, axis), exact, rtol=1e-12, atol=1e-14)


def test_one_rebased_iteration_is_one_plain_iteration():
    rng = np.random.default_rng(2)
    shape = (10, 8)
    dt, sig = 0.2, (0.7, 1.3)
    Hold = 1.0 + rng.random(shape)
    Hb = Hold + 0.01 * rng.standard_normal(shape)
    d = 1e-3 * rng.standard_normal(shape)
    wb = [rng.standard_normal((shape[0] - 1, shape[1])), rng.standard_normal((shape[0], shape[1] - 1))]
    om = [1e-3 * rng.standard_normal(w.shape) for w in wb]
    c = [0.3 + 0.5 * rng.random(w.shape) for w in wb]        # per-face iteration parameters
    e = 0.05 + 0.05 * rng.random(shape)                       # per-cell iteration parameter

    # plain iteration on the summed state
    H = Hb + d
    w = [wb[k] + om[k] for k in range(2)]
    w_new = [w[k] - c[k] * (w[k] + u_nonlin(H, k)) for k in range(2)]
    R = (H - Hold) / dt + sum(div(w_new[k], k, shape) * sig[k] for k in range(2))
    H_new = H.copy()
    H_new[1:-1, 1:-1] = (H - e * R)[1:-1, 1:-1]

    # rebased iteration on the change
    tb = [wb[k] + u_nonlin(Hb, k) for k in range(2)]
    om_new = [om[k] - c[k] * (tb[k] + om[k] + u_delta(Hb, d, k)) for k in range(2)]
    Rb = (Hb - Hold) / dt + sum(div(wb[k], k, shape) * sig[k] for k in range(2))
    Rd = Rb + d / dt + sum(div(om_new[k], k, shape) * sig[k] for k in range(2))
    d_new = d.copy()
    d_new[1:-1, 1:-1] = (d - e * Rd)[1:-1, 1:-1]

    for k in range(2):
        assert np.allclose(wb[k] + om_new[k], w_new[k], rtol=1e-12, atol=1e-13)
    assert np.allclose(Hb + d_new, H_new, rtol=1e-13, atol=1e-13)


def test_base_residual_vanishes_at_a_fixed_point():
    """At a fixed point of the plain iteration (w = -u(H), R = 0) the rebased
    form with delta = omega = 0 has t_b = 0 and R_b = 0: it stays put."""
    rng = np.random.default_rng(3)
    shape = (8, 6)
    Hb = 1.0 + rng.random(shape)
    wb = [-u_nonlin(Hb, k) for k in range(2)]
    tb = [wb[k] + u_nonlin(Hb, k) for k in range(2)]
    assert all(np.max(np.abs(t)) == 0.0 for t in tb)


def test_defect_correction_jacobian_is_the_linear_part():
    """The FP32_DC inner iteration applies the linearised flux
    J d = 3 s^2 g (d_L + d_R) + s^3 (d_R - d_L) (ptd_dc_body.cuh, face32):
    u(H_b + eps d) - u(H_b) - eps J d shrinks like eps^2."""
    rng = np.random.default_rng(4)
    Hb = 1.0 + rng.random((9, 7))
    d = rng.standard_normal((9, 7))
    for axis in (0, 1):
        L, R = faces(Hb, axis)
        dL, dR = faces(d, axis)
        s, g = L + R, R - L
        Jd = 3 * s ** 2 * g * (dL + dR) + s ** 3 * (dR - dL)
        rem = [np.max(np.abs(u_delta(Hb, eps * d, axis) - eps * Jd)) for eps in (1e-2, 1e-3)]
        assert rem[1] < rem[0] / 50   # ~ eps^2: a 10x smaller eps gives ~100x smaller remainder
