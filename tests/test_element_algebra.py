"""The mixed path's element algebra (element_mixed_kernel, kernels_element_mixed.cuh), restated in numpy FP64 and
checked against the reference's element forces from the oracle (the C restatement pinned bit-exact to the
reference build).

The mixed kernel does not evaluate the reference's expressions in the reference's order; it rearranges them so
that FP32 loses nothing to cancellation near the rest state:

* K = I + J0^-1 dU from the vertices' displacements from rest (the reference's J_inv_0 J), vol = vol_0 det K and
  J^-1 = K^-1 J0^-1 (calculate_jacobian / calc_shape_function_derivatives_and_volume,
  src/tetra_element_linear.cpp:191-292);
* shear + bulk stress = (G / det K)(M + M^T + M M^T) + (E - 2G/3)(det K - 1)(det K + 1)/(2 det K) I with
  M = K^T - I (add_shear_elastic_stress + add_bulk_elastic_stress, :375-403);
* the inertial viscous force V_e v_e (get_element_velocity_vector + mat12_apply, :448-463) as the stress
  B tr(L) I + A (L + L^T) of the velocity gradient L.

Evaluated in FP64 these must reproduce the reference's node forces to rounding (1e-11 of the largest), which pins
the rearrangement itself; the GPU tests then bound what FP32 adds.
"""
import numpy as np

import pyoracle as po
from gen_golden import case_mesh, sheared


def mixed_element_forces(x, v, rest, tets4, jinv0, vol0, mat):
    """Node forces (T, 4, 3) of the rearranged algebra at positions x and velocities v (vertices, meso units)."""
    u = x - rest
    dU = u[tets4[:, 1:]] - u[tets4[:, :1]]                        # (T, 3, 3): rows = edge displacements
    Kd = np.einsum("trk,tkc->trc", jinv0, dU)                      # J0^-1 dU
    tr = np.trace(Kd, axis1=1, axis2=2)
    minors = (Kd[:, 0, 0] * Kd[:, 1, 1] - Kd[:, 0, 1] * Kd[:, 1, 0] + Kd[:, 0, 0] * Kd[:, 2, 2]
              - Kd[:, 0, 2] * Kd[:, 2, 0] + Kd[:, 1, 1] * Kd[:, 2, 2] - Kd[:, 1, 2] * Kd[:, 2, 1])
    delta = tr + minors + np.linalg.det(Kd)
    dK = 1.0 + delta
    K = np.eye(3) + Kd
    Jinv = np.einsum("tjk,tkm->tjm", np.linalg.inv(K), jinv0)     # J^-1 = K^-1 J0^-1
    grad = np.zeros((len(tets4), 3, 4))                            # grad[t, j, a] = d psi_a / d x_j
    grad[:, :, 1:] = Jinv
    grad[:, :, 0] = -Jinv.sum(axis=2)
    vol = vol0 * dK
    A, B, G, E = mat[:, 1], mat[:, 2], mat[:, 3], mat[:, 4]
    M = np.transpose(Kd, (0, 2, 1))
    S = (G / dK)[:, None, None] * (M + np.transpose(M, (0, 2, 1)) + np.einsum("tik,tjk->tij", M, M))
    c2 = E - G * 2.0 / 3.0
    S += (0.5 * c2 * delta * (2.0 + delta) / dK)[:, None, None] * np.eye(3)
    L = np.einsum("tbi,tjb->tij", v[tets4], grad)                  # velocity gradient
    S += (B * np.trace(L, axis1=1, axis2=2))[:, None, None] * np.eye(3)
    S += A[:, None, None] * (L + np.transpose(L, (0, 2, 1)))
    return -vol[:, None, None] * np.einsum("tja,tij->tai", grad, S)


def test_rearranged_element_algebra_matches_reference(oracle_built):
    m = case_mesh(4, 5)
    o = po.OracleBlob(m, solver="masslumped", dt=1e-14, kT=0.0, calc_noise=0, threads=1)
    rest = o.pos()
    o.set_pos(sheared(m, 0.03))
    assert o.step(5) == 0  # velocities of the mass-lumped dynamics
    o.zero_forces()
    assert o.update_internal_forces() == 0
    e = o.elem()
    r = o.rest()
    tets4 = np.asarray(m.tets)[:, :4]
    x, v = o.pos(), o.vel()
    got = mixed_element_forces(x, v, rest, tets4, r["jinv0"], e["vol0"], r["mat"])
    want = e["node_force"][:, :4, :]
    scale = np.abs(want).max()
    assert scale > 0 and np.abs(v).max() > 0
    err = np.abs(got - want).max() / scale
    print(f"rearranged element algebra vs the reference's node forces: {err:.2e} of the largest")
    assert err < 1e-11
