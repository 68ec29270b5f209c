"""The algebra of the mixed path's residual-row kernel (fluid_res_dw_kernel in
csrc/k_fluid.cu), restated in FP64 numpy and checked against the oracle's element
integrand (pyoracle.fluid_element, the reference's fluid_3d_m / fluid_3d_c,
fluid.cpp:1389-2139) on random elements and states.

The kernel regroups the integrand for the P1 tet and its symmetric 4-point rule
(N_g(a) = s for a = g, t otherwise, s + 3t = 1):
  * velocity and pressure gradients, div u and the viscous part of RM are element
    constants;
  * a Gauss-point value is t * (sum over the nodes) + (s - t) * (the value at node g);
  * sum_g N_g(a) v_g = t * (sum over the points) + (s - t) * v_a, so RV needs one sum
    and the per-point rV2; sum_g N_g(a) div u = SN div u; sum_g up_g . grad N_a =
    (sum_g up_g) . grad N_a; sum_g p_g = SN * (sum over the nodes).
These are identities of real arithmetic; here they hold to FP64 rounding (1e-12
relative per element), which the GPU test of the double-word kernel then tightens to
the kernel's own arithmetic."""
import numpy as np
import pytest

from oracle import pyoracle as po


def regrouped_rows(P, xl, al, yl):
    """lR[a, i] of one element by the kernel's regrouped formula, FP64."""
    qs = (5.0 + 3.0 * np.sqrt(5.0)) / 20.0
    qt = (1.0 - qs) / 3.0
    SN = qs + 3.0 * qt
    rho, mu, kd, dt = P.rho, P.mu, P.k_inv_darcy, P.dt
    f = np.array([P.fx, P.fy, P.fz])
    J = np.stack([xl[0] - xl[3], xl[1] - xl[3], xl[2] - xl[3]], axis=1)  # J[i, j] = dx_i / dxi_j
    Jac = np.linalg.det(J)
    xiX = np.linalg.inv(J)  # xiX[j, k] = dxi_j / dx_k
    Nx = np.zeros((3, 4))
    Nx[:, :3] = xiX.T
    Nx[:, 3] = -xiX.sum(axis=0)
    K = xiX.T @ xiX
    w = Jac / 24.0
    mur = mu / rho
    kTS = 4.0 / dt ** 2 + (kd * mur) ** 2 + 36.0 * np.sum(K * K) * mur ** 2
    trK = np.trace(K)
    y, a, p = yl[:, :3], al[:, :3], yl[:, 3]
    ux = Nx @ y           # ux[k, i] = du_i / dx_k
    px = Nx @ p
    divU = np.trace(ux)
    Cy, Cp, Ca = qt * y.sum(0), qt * p.sum(), qt * a.sum(0) - f
    RM = 4.0 * mu * (ux + ux.T)
    SrV2, Sup, sTauC = np.zeros(3), np.zeros(3), 0.0
    rV2s = np.zeros((4, 3))
    for g in range(4):
        u = Cy + (qs - qt) * y[g]
        ud = Ca + (qs - qt) * a[g]
        tauM = 1.0 / (rho * np.sqrt(kTS + u @ K @ u))
        up = -tauM * (rho * (ud + u @ ux) + px + mu * kd * u)
        sTauC += 1.0 / (tauM * trK)
        tauB = up @ K @ up
        if abs(tauB) < 10.0 * 2.0 ** -104:
            tauB = 2.0 ** -52
        tauB = rho / np.sqrt(tauB)
        ua = u + up
        rVb = tauB * (up @ ux)
        RM += np.outer(up, rVb) - np.outer(ua, rho * up)   # RM[k, i] += rVb_i up_k - rho up_i ua_k
        rV2 = rho * (ud + ua @ ux) + mu * kd * ua
        SrV2 += rV2
        rV2s[g] = rV2
        Sup += up
    RM[np.diag_indices(3)] += divU * sTauC - SN * p.sum()
    lR = np.zeros((4, 4))
    for aa in range(4):
        RV = qt * SrV2 + (qs - qt) * rV2s[aa]
        lR[aa, :3] = w * (RV + Nx[:, aa] @ RM)
        lR[aa, 3] = w * (SN * divU - Sup @ Nx[:, aa])
    return lR


@pytest.mark.parametrize("kd", [0.0, 0.3])
def test_regrouped_rows_match_the_reference_integrand(kd):
    rng = np.random.default_rng(11)
    P = po.fluid_params(k_inv_darcy=kd, f=(0.1, -0.2, 0.05))
    worst = 0.0
    for _ in range(300):
        # a random, well-shaped tet around the unit simplex, random state
        xl = np.array([[1.0, 0, 0], [0, 1.0, 0], [0, 0, 1.0], [0, 0, 0]]) * rng.uniform(0.05, 0.2)
        xl = xl + 0.02 * rng.standard_normal((4, 3)) + rng.standard_normal(3)
        al = rng.standard_normal((4, 4))
        yl = rng.standard_normal((4, 4)) * np.array([10.0, 10.0, 10.0, 50.0])
        ref, _ = po.fluid_element(P, xl, al, yl)
        got = regrouped_rows(P, xl, al, yl)
        worst = max(worst, float(np.abs(got - ref).max() / np.abs(ref).max()))
    print("max relative difference over 300 elements:", worst)
    assert worst <= 1e-12
