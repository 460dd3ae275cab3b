"""Test infrastructure: a numpy restatement of the device SCF's density step
(hartree_fock_cpp_gb300/csrc/hfx_sp2.cu), step for step: Gershgorin bounds of
sym(F), X_0 = (e_max I - F) / (e_max - e_min), then per step the branch
X <- X^2 if |tr X^2 - n_occ| < |2 tr X - tr X^2 - n_occ| else 2X - X^2, the
stop two steps after tr X - tr X^2 first falls below 1e-10, and the final
trace check.  The kernels follow this control exactly; the host tests check
the control itself against an eigendecomposition."""
import numpy as np

IDEM_TOL = 1e-10
TRACE_TOL = 1e-6


def sp2_projector(F, nocc, max_steps=100):
    """(D, steps) with steps = the status word (answer step + 1), or (None, 0)."""
    F = 0.5 * (F + F.T)
    n = F.shape[0]
    r = np.abs(F).sum(1) - np.abs(np.diag(F))
    lo, hi = (np.diag(F) - r).min(), (np.diag(F) + r).max()
    X = (hi * np.eye(n) - F) * (1.0 / (hi - lo))
    Xs = [X]
    X2s = [X @ X]
    kstar, answer = -1, -1
    for j in range(1, max_steps + 1):           # the decision before step j (j == max_steps: the finishing kernel)
        sx, sx2 = np.trace(Xs[j - 1]), np.trace(X2s[j - 1])
        if kstar < 0 and sx - sx2 < IDEM_TOL:
            kstar = j - 1
        if kstar >= 0 and j - 1 >= kstar + 2:
            answer = j - 1
            break
        if j == max_steps:
            break
        X = X2s[j - 1] if abs(sx2 - nocc) < abs(2 * sx - sx2 - nocc) else 2 * Xs[j - 1] - X2s[j - 1]
        Xs.append(X)
        X2s.append(X @ X)
    if answer < 0 or not abs(np.trace(Xs[answer]) - nocc) < TRACE_TOL:
        return None, 0
    return Xs[answer], answer + 1
