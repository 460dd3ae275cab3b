"""numpy restatement of the kernels' per-shell-quartet arithmetic (stage 1 R
recursion, stage 2 ket transform, stage 3 bra transform) over the host image
of the pair data (hfx_debug_pair_data).  Test infrastructure: it checks on
the CPU that the pair data the kernels read encodes the reference's ERIs."""
import ctypes
import math

import numpy as np

import oracle as O
from hartree_fock_cpp_gb300 import _lib


def nherm(L):
    return (L + 1) * (L + 2) * (L + 3) // 6


def ncart(l):
    return (l + 1) * (l + 2) // 2


def herm_comps(L):
    return [(t, u, s - t - u) for s in range(L + 1) for t in range(s + 1) for u in range(s - t + 1)]


def herm_index(t, u, v):
    s = t + u + v
    return s * (s + 1) * (s + 2) // 6 + t * (s + 1) - t * (t - 1) // 2 + u


def pair_data(config, basis_set):
    m = _lib.MoleculeArgs(config, basis_set)
    n1, n2, n3 = ctypes.c_int(), ctypes.c_int(), ctypes.c_longlong()
    _lib.check(_lib.lib.hfx_debug_pair_data(m.ref(), ctypes.byref(n1), ctypes.byref(n2), ctypes.byref(n3), None,
                                            None, None))
    rec = np.zeros(10 * n1.value, np.int32)
    geo = np.zeros(4 * n2.value)
    ep = np.zeros(n3.value)
    _lib.check(_lib.lib.hfx_debug_pair_data(m.ref(), None, None, None, _lib.ptr(rec), _lib.ptr(geo), _lib.ptr(ep)))
    return rec.reshape(-1, 10), geo.reshape(-1, 4), ep


def hermite_R(L, p, q, X, Y, Z):
    rho = p * q / (p + q)
    T = rho * (X * X + Y * Y + Z * Z)
    bo = O.lib()
    seeds = [(-2 * rho) ** m * bo.orc_boys_stable(m, T) for m in range(L + 1)]
    prev = {(0, 0, 0): seeds[L]}
    for n in range(L - 1, -1, -1):
        cur = {}
        for (t, u, v) in herm_comps(L - n):
            if t + u + v == 0:
                val = seeds[n]
            elif t > 0:
                val = X * prev[(t - 1, u, v)] + ((t - 1) * prev[(t - 2, u, v)] if t > 1 else 0.0)
            elif u > 0:
                val = Y * prev[(t, u - 1, v)] + ((u - 1) * prev[(t, u - 2, v)] if u > 1 else 0.0)
            else:
                val = Z * prev[(t, u, v - 1)] + ((v - 1) * prev[(t, u, v - 2)] if v > 1 else 0.0)
            cur[(t, u, v)] = val
        prev = cur
    return prev


def shell_quartet_block(rec, geo, ep, bra, ket):
    b, k = rec[bra], rec[ket]
    L1, L2 = b[2] + b[3], k[2] + k[3]
    H1, H2 = nherm(L1), nherm(L2)
    nab, ncd = ncart(b[2]) * ncart(b[3]), ncart(k[2]) * ncart(k[3])
    eb, ek = int(b[6]) + (int(b[7]) << 32), int(k[6]) + (int(k[7]) << 32)
    cb, ck = herm_comps(L1), herm_comps(L2)
    acc = np.zeros((nab, ncd))
    for ij in range(b[5]):
        g1 = geo[b[4] + ij]
        Eij = ep[eb + ij * nab * H1: eb + (ij + 1) * nab * H1].reshape(nab, H1)
        for kl in range(k[5]):
            g2 = geo[k[4] + kl]
            Ekl = ep[ek + kl * ncd * H2: ek + (kl + 1) * ncd * H2].reshape(ncd, H2)
            p, q = g1[0], g2[0]
            R = hermite_R(L1 + L2, p, q, g1[1] - g2[1], g1[2] - g2[2], g1[3] - g2[3])
            pref = 2 * math.pi ** 2.5 / (p * q * math.sqrt(p + q))
            M = np.array([[(-1) ** (a + bb + c) * R[(t + a, u + bb, v + c)] for (a, bb, c) in ck]
                          for (t, u, v) in cb])
            acc += pref * Eij @ M @ Ekl.T
    return acc
