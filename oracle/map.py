"""Float64 restatement of the MAP objective (test infrastructure: only tests/ use it).

The reference has no MAP path; its OSEM weights (recon_osem_plane.py:28-42) are the
likelihood's gradient plus the sensitivity, and that is what the projector halves are tested
against. This file restates, in float64 and independently of the kernels' algebra:

* the relative-difference prior (Nuyts et al., IEEE Trans. Nucl. Sci. 49(1):56-60, 2002)
  R(x) = sum over undirected edges {j, k} of w_jk (x_j - x_k)^2 / (x_j + x_k + gamma|x_j - x_k| + eps),
  each edge once (the table holds both directions), gradient by the quotient rule;
* the Poisson log-likelihood of SC projections with rotations (f[b, r] = A[b] . x[rot[:, r] - 1],
  recon_osem_plane.py:51 gathers the rotated image the same way) and of list-mode Compton
  events (g = T x, minus the Compton sensitivity s_c . x);
* the log-parameterised objective Phi(z) = -L(e^z) + beta R(e^z) and its z-gradient.

Gradients here are checked against float64 central differences (tests/test_map_oracle.py),
so the restatement is pinned by calculus rather than by reference outputs.
"""
from __future__ import annotations

import numpy as np


def table_edges(nbr, weight):
    """Undirected edges (j, k, w) with j < k of a neighbour-major table [K, V]."""
    nbr = np.asarray(nbr)
    weight = np.asarray(weight, dtype=np.float64)
    K, V = nbr.shape
    j = np.broadcast_to(np.arange(V)[None, :], (K, V))
    m = (nbr >= 0) & (j < nbr)
    return j[m].astype(np.int64), nbr[m].astype(np.int64), weight[m]


def rdp(x, nbr, weight, gamma, eps=1e-9):
    """(R(x), dR/dx) in float64."""
    x = np.asarray(x, dtype=np.float64).ravel()
    j, k, w = table_edges(nbr, weight)
    a, b = x[j], x[k]
    d = a - b
    den = a + b + gamma * np.abs(d) + eps
    value = float(np.sum(w * d * d / den))
    # quotient rule on phi = d^2 / den: d(den)/da = 1 + gamma sgn(d), d(den)/db = 1 - gamma sgn(d)
    sg = np.sign(d)
    da = w * (2 * d * den - d * d * (1 + gamma * sg)) / den ** 2
    db = w * (-2 * d * den - d * d * (1 - gamma * sg)) / den ** 2
    grad = np.zeros_like(x)
    np.add.at(grad, j, da)
    np.add.at(grad, k, db)
    return value, grad


def sc_log_likelihood(x, A, y, rot=None):
    """(L_SC(x), dL_SC/dx): sum_{b,r} y log f - f with f[b, r] = A[b] . x[rot[:, r] - 1]."""
    x = np.asarray(x, dtype=np.float64).ravel()
    A = np.asarray(A, dtype=np.float64)
    y = np.asarray(y, dtype=np.float64).reshape(A.shape[0], -1)
    R = y.shape[1]
    value, grad = 0.0, np.zeros_like(x)
    for r in range(R):
        idx = np.arange(x.size) if rot is None else np.asarray(rot)[:, r].astype(np.int64) - 1
        f = A @ x[idx]
        value += float(np.sum(y[:, r] * np.log(f) - f))
        np.add.at(grad, idx, A.T @ (y[:, r] / f - 1.0))
    return value, grad


def compton_log_likelihood(x, T, s_c):
    """(L_C(x), dL_C/dx): sum_i log (T x)_i - s_c . x."""
    x = np.asarray(x, dtype=np.float64).ravel()
    T = np.asarray(T, dtype=np.float64)
    s = np.asarray(s_c, dtype=np.float64).ravel()
    g = T @ x
    return float(np.sum(np.log(g)) - s @ x), T.T @ (1.0 / g) - s


def map_objective(z, sc=None, compton=None, prior=None):
    """(Phi(z), dPhi/dz) with x = exp(z): Phi = -L_SC - L_C + beta R.
    sc = (A, y, rot); compton = (T, s_c); prior = (nbr, weight, beta, gamma, eps)."""
    z = np.asarray(z, dtype=np.float64).ravel()
    x = np.exp(z)
    value, gx = 0.0, np.zeros_like(x)
    if sc is not None:
        v, g = sc_log_likelihood(x, *sc)
        value -= v
        gx -= g
    if compton is not None:
        v, g = compton_log_likelihood(x, *compton)
        value -= v
        gx -= g
    if prior is not None:
        nbr, weight, beta, gamma, eps = prior
        v, g = rdp(x, nbr, weight, gamma, eps)
        value += beta * v
        gx += beta * g
    return value, gx * x


def adam(grad_fn, z0, lr, n_steps, beta1=0.9, beta2=0.999, eps=1e-8):
    """Adam (Kingma & Ba, ICLR 2015, Algorithm 1 with bias correction) on grad_fn(z) ->
    (value, grad); returns (z, values before each step)."""
    z = np.asarray(z0, dtype=np.float64).copy()
    m = np.zeros_like(z)
    v = np.zeros_like(z)
    hist = []
    for t in range(1, n_steps + 1):
        val, g = grad_fn(z)
        hist.append(val)
        m = beta1 * m + (1 - beta1) * g
        v = beta2 * v + (1 - beta2) * g * g
        mh = m / (1 - beta1 ** t)
        vh = v / (1 - beta2 ** t)
        z = z - lr * mh / (np.sqrt(vh) + eps)
    return z, np.array(hist)
