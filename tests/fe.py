"""Small-strain linear elasticity of a blob's vertex nodes, as a yardstick for the physics tests.

The reference's shear and bulk stresses (tetra_element_linear::add_shear_elastic_stress and
add_bulk_elastic_stress, src/tetra_element_linear.cpp:375-403) linearise about the rest state to
isotropic linear elasticity with Lame constants mu = G and lambda = K - 2G/3 (G the shear modulus, K the
bulk modulus). The stiffness matrix of the linear tetrahedra on the vertex nodes gives the static response
to a load and, at temperature T, the Boltzmann variance kT / lambda_k of each normal mode.
"""
import numpy as np


def linear_stiffness(pos_m, tets4, G, K):
    """Stiffness matrix (3 Nv x 3 Nv, N/m, scipy CSR) of linear tetrahedra with vertex positions pos_m (m)."""
    import scipy.sparse as sp
    G = np.broadcast_to(np.asarray(G, float), (tets4.shape[0],))
    K = np.broadcast_to(np.asarray(K, float), (tets4.shape[0],))
    nv = pos_m.shape[0]
    rows, cols, vals = [], [], []
    for e in range(tets4.shape[0]):
        lam = K[e] - 2.0 * G[e] / 3.0
        D = np.zeros((6, 6))
        D[:3, :3] = lam
        D[np.arange(3), np.arange(3)] += 2.0 * G[e]
        D[np.arange(3, 6), np.arange(3, 6)] = G[e]
        Mx = np.hstack([np.ones((4, 1)), pos_m[tets4[e]]])
        g = np.linalg.inv(Mx)[1:, :]
        V = abs(np.linalg.det(Mx)) / 6.0
        B = np.zeros((6, 12))
        for a in range(4):
            gx, gy, gz = g[:, a]
            B[0, 3 * a], B[1, 3 * a + 1], B[2, 3 * a + 2] = gx, gy, gz
            B[3, 3 * a], B[3, 3 * a + 1] = gy, gx
            B[4, 3 * a + 1], B[4, 3 * a + 2] = gz, gy
            B[5, 3 * a], B[5, 3 * a + 2] = gz, gx
        idx = (3 * tets4[e][:, None] + np.arange(3)).ravel()
        rows.append(np.repeat(idx, 12))
        cols.append(np.tile(idx, 12))
        vals.append((V * B.T @ D @ B).ravel())
    return sp.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))), shape=(3 * nv,) * 2)


def linear_fe_extension(mesh, f_ext, pinned, G, K):
    """Static displacement (m) of every vertex under the vertex forces f_ext (N), pinned vertices held."""
    import scipy.sparse.linalg as spla
    nv = mesh.n_linear
    Kg = linear_stiffness(mesh.pos[:nv] * mesh.scale, mesh.tets[:, :4], G, K)
    free = np.ones(3 * nv, bool)
    pv = pinned[pinned < nv]
    for c in range(3):
        free[3 * pv + c] = False
    u = np.zeros(3 * nv)
    u[free] = spla.spsolve(Kg[free][:, free].tocsc(), f_ext[:nv].ravel()[free])
    return u.reshape(-1, 3)


def mode_variance_ratios(frames_m, rest_m, tets4, G, K, kT):
    """Per internal normal mode k of the stiffness at rest_m: the sample variance of the mode amplitude over the
    frames (F, Nv, 3; m), divided by the Boltzmann value kT / lambda_k, and the number of effectively
    independent samples of each amplitude (from its integrated autocorrelation time)."""
    Kd = linear_stiffness(rest_m, tets4, G, K).toarray()
    lam, phi = np.linalg.eigh(0.5 * (Kd + Kd.T))
    keep = lam > 1e-8 * lam.max()  # drops the six rigid-body modes
    u = frames_m.reshape(frames_m.shape[0], -1)
    u = u - u.mean(axis=0)
    a = u @ phi[:, keep]
    var = a.var(axis=0)
    ratio = var * lam[keep] / kT
    F = a.shape[0]
    neff = np.empty(a.shape[1])
    for k in range(a.shape[1]):
        x = a[:, k] / np.sqrt(var[k])
        tau = 1.0
        for lag in range(1, F // 4):
            rho = float(np.mean(x[:-lag] * x[lag:]))
            if rho < 0.05:
                break
            tau += 2.0 * rho
        neff[k] = F / tau
    return ratio, neff
