"""Numpy restatement of the leap-frog adjoint of lq_leapfrog_adjoint, for small lattices.

Test infrastructure only.  The adjoint has no counterpart in the reference crate; its forward
states come from the oracle's restatement of the reference's force (derivative_e,
src/simulation/state.rs:1420-1448) and link derivative (derivative_u, :1407-1417), and the
cotangent recursion is the one documented in csrc/adjoint.cuh:
  adj drift : lam_E^a += -kappa Im Tr(T^a U lam_U^dag),  lam_U <- lam_U - kappa i E lam_U
  adj kick  : lam_U += h c d/dU sum_l Im Tr(W_l U_l Sigma_l),  W_l = sum_a lam_E^a T^a
with c = -sqrt(2/3)/size, kappa = dt sqrt(6)/size, O = Re average_trace_plaquette / 3."""
import numpy as np


def geometry(dim, L):
    V = L ** dim
    coords = np.array([(s // L ** i) % L for s in range(V) for i in range(dim)]).reshape(V, dim)
    strides = np.array([L ** i for i in range(dim)])
    fwd = np.zeros((V, dim), dtype=np.int64)
    bwd = np.zeros((V, dim), dtype=np.int64)
    for mu in range(dim):
        cp = coords.copy()
        cp[:, mu] = (cp[:, mu] + 1) % L
        fwd[:, mu] = cp @ strides
        cm = coords.copy()
        cm[:, mu] = (cm[:, mu] - 1) % L
        bwd[:, mu] = cm @ strides
    return V, fwd, bwd


def to_mats(O, links, dim, L):
    V = L ** dim
    return np.array([O.to_complex(m) for m in links]).reshape(V, dim, 3, 3)


def from_mats(O, U):
    return np.array([O.from_complex(m) for m in U.reshape(-1, 3, 3)])


def generators(O):
    return np.array([O.to_complex(g) for g in O.generators()])


def staple_sum(U, fwd, bwd, x, mu):
    dim = U.shape[1]
    s = np.zeros((3, 3), dtype=complex)
    for nu in range(dim):
        if nu == mu:
            continue
        xpmu, xpnu, xmnu = fwd[x, mu], fwd[x, nu], bwd[x, nu]
        s += U[xpmu, nu] @ U[xpnu, mu].conj().T @ U[x, nu].conj().T
        s += U[bwd[xpmu, nu], nu].conj().T @ U[xmnu, mu].conj().T @ U[xmnu, nu]
    return s


def _loop_r(factors, wm):
    """R of a loop U_m X Y Z; factors: (U_l, W_l, forward)."""
    p = q = None
    for u, w, f in factors:
        x = u if f else u.conj().T
        d = w @ u if f else -(u.conj().T @ w)
        if p is None:
            p, q = x, d
        else:
            p, q = p @ x, q @ x + p @ d
    return q + p @ wm


def adj_kick(U, lamE, lamU, coef, T, fwd, bwd):
    V, dim = U.shape[:2]
    W = np.einsum("xma,aij->xmij", lamE, T)
    out = lamU.copy()
    for x in range(V):
        for mu in range(dim):
            r = np.zeros((3, 3), dtype=complex)
            xpmu = fwd[x, mu]
            for nu in range(dim):
                if nu == mu:
                    continue
                xpnu, xmnu = fwd[x, nu], bwd[x, nu]
                r += _loop_r([(U[xpmu, nu], W[xpmu, nu], True), (U[xpnu, mu], W[xpnu, mu], False),
                              (U[x, nu], W[x, nu], False)], W[x, mu])
                y = bwd[xpmu, nu]
                r += _loop_r([(U[y, nu], W[y, nu], False), (U[xmnu, mu], W[xmnu, mu], False),
                              (U[xmnu, nu], W[xmnu, nu], True)], W[x, mu])
            out[x, mu] += coef * 1j * r.conj().T
    return out


def adj_drift(U, E, lamU, lamE, kappa, T):
    Ehat = np.einsum("xma,aij->xmij", E, T)
    prod = U @ lamU.conj().transpose(0, 1, 3, 2)
    lamE = lamE - kappa * np.einsum("aij,xmji->xma", T, prod).imag
    lamU = lamU - kappa * 1j * (Ehat @ lamU)
    return lamU, lamE


def leapfrog_adjoint(O, dim, L, size, links, efield, dt, n):
    """objective, dO/dU0 [V, D, 3, 3] complex, dO/dE0 [V, D, 8]"""
    T = generators(O)
    V, fwd, bwd = geometry(dim, L)
    c = -np.sqrt(2.0 / 3.0) / size
    kappa = dt * np.sqrt(6.0) / size
    us, es = [], []  # U_k and the momenta after kick k
    u, e = links.copy(), efield.copy()
    for k in range(n):
        h = dt / 2.0 if k == 0 else dt
        # kick k: the end kick of step k-1 and the start kick of step k (dt/2 + dt/2)
        e = e + h * O.derivative_e(dim, L, size, u)
        us.append(u)
        es.append(e)
        u = u + dt * O.derivative_u(dim, L, size, u, e)
    n_plaq = V * dim * (dim - 1) // 2
    objective = O.average_trace_plaquette(dim, L, u).real / 3.0
    Un = to_mats(O, u, dim, L)
    lamU = np.zeros_like(Un)
    for x in range(V):
        for mu in range(dim):
            lamU[x, mu] = staple_sum(Un, fwd, bwd, x, mu).conj().T / (3.0 * n_plaq)
    lamE = np.zeros((V, dim, 8))
    for k in range(n - 1, -1, -1):
        Uk = to_mats(O, us[k], dim, L)
        lamU, lamE = adj_drift(Uk, es[k].reshape(V, dim, 8), lamU, lamE, kappa, T)
        h = dt / 2.0 if k == 0 else dt
        lamU = adj_kick(Uk, lamE, lamU, h * c, T, fwd, bwd)
    return objective, lamU, lamE


def objective(O, dim, L, size, links, efield, dt, n):
    u, _ = O.integrate(dim, L, size, links, efield, O.SYMPLECTIC, dt, n)
    return O.average_trace_plaquette(dim, L, u).real / 3.0
