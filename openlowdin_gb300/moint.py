"""The reference's transformed-integral file `<species>moint.dat`.

Layout (TransformIntegralsC.f90:531-654 writes it, ReadTransformedIntegrals.f90:225-233
reads it): Fortran sequential unformatted records, each framed by its length
in bytes (int32) before and after, holding four int32 index arrays p, q, r, s
(1-based orbital numbers) and one FP64 value array, all of the stack size
(CONTROL's INTEGRAL_STACK_SIZE, 30000 by default).  The last record marks the
end with p = -1 after its last entry.

For the MP2 transform of one species the entries are (ia|jb) in the order
p = i, q = a, r = j >= i, s = b (b >= a when j == i), |value| > 1e-10
(LowdinGB300_mp2_moint); for a species pair every i, a of the first and j, b
of the second species in that order (LowdinGB300_mp2_coupling_moint).  This
module reads them back and evaluates the MP2 terms from them as
MPFunctions.f90:514-662 (closed shell) and :682-886 (inter-species) do.
"""
from __future__ import annotations

import numpy as np


def read_moint(path: str, stack_size: int = 30000):
    """(p, q, r, s, values) of every entry of the file, in file order."""
    rec = stack_size * (4 * 4 + 8)
    out = [[], [], [], [], []]
    with open(path, "rb") as f:
        while True:
            head = f.read(4)
            if len(head) < 4:
                raise ValueError(f"{path}: no end marker (p = -1) before the end of the file")
            n = int(np.frombuffer(head, np.int32)[0])
            if n != rec:
                raise ValueError(f"{path}: record of {n} bytes, expected {rec} (stack size {stack_size})")
            body = f.read(rec)
            tail = f.read(4)
            if len(body) < rec or len(tail) < 4 or int(np.frombuffer(tail, np.int32)[0]) != rec:
                raise ValueError(f"{path}: truncated or unframed record")
            idx = np.frombuffer(body, np.int32, 4 * stack_size).reshape(4, stack_size)
            val = np.frombuffer(body, np.float64, stack_size, offset=16 * stack_size)
            end = np.flatnonzero(idx[0] == -1)
            m = int(end[0]) if end.size else stack_size
            for k in range(4):
                out[k].append(idx[k, :m].copy())
            out[4].append(val[:m].copy())
            if end.size:
                break
    return tuple(np.concatenate(x) if x else np.zeros(0) for x in out)


def mp2_entries(iajb, n_frozen: int, n_occ: int, cut: float = 1e-10):
    """Entries of the file for a full (ia|jb) tensor iajb[i, a, j, b] over the
    active occupied (i, j) and virtual (a, b) orbitals, in the writer's order."""
    o, v = iajb.shape[0], iajb.shape[1]
    P, Q, R, S, V = [], [], [], [], []
    for i in range(o):
        for a in range(v):
            for j in range(i, o):
                b0 = a if j == i else 0
                vals = iajb[i, a, j, b0:]
                keep = np.flatnonzero(np.abs(vals) > cut)
                P += [n_frozen + i + 1] * len(keep)
                Q += [n_occ + a + 1] * len(keep)
                R += [n_frozen + j + 1] * len(keep)
                S += list(n_occ + b0 + keep + 1)
                V += list(vals[keep])
    return (np.asarray(P, np.int32), np.asarray(Q, np.int32), np.asarray(R, np.int32), np.asarray(S, np.int32),
            np.asarray(V, np.float64))


def mp2_energy(entries, eps, n_occ: int, n_frozen: int, n_basis: int) -> float:
    """Closed-shell E_MP2 = sum_{ijab} (ia|jb) [2 (ia|jb) - (ib|ja)] /
    (e_i + e_j - e_a - e_b) from the file's unique entries ((ia|jb) = (jb|ia);
    absent entries are zero)."""
    p, q, r, s, v = entries
    o, nv = n_occ - n_frozen, n_basis - n_occ
    T = np.zeros((o, nv, o, nv))
    i, a, j, b = p - 1 - n_frozen, q - 1 - n_occ, r - 1 - n_frozen, s - 1 - n_occ
    T[i, a, j, b] = v
    T[j, b, i, a] = v
    e = np.asarray(eps, np.float64)
    eo, ev = e[n_frozen:n_occ], e[n_occ:n_basis]
    D = eo[:, None, None, None] - ev[None, :, None, None] + eo[None, None, :, None] - ev[None, None, None, :]
    return float(np.sum(T * (2.0 * T - T.transpose(0, 3, 2, 1)) / D))


def mp2_coupling_energy(entries, eps_a, eps_b, factor: float) -> float:
    """Inter-species MP2 term from a two-species file (every (ia|jb) with i, a
    of species a and j, b of species b; absent entries are zero):
    factor * sum (ia|jb)^2 / (e_i + e_j - e_a - e_b), factor = (q_a q_b)^2
    lambda_a lambda_b (MPFunctions.f90:682-886)."""
    p, q, r, s, v = entries
    ea, eb = np.asarray(eps_a, np.float64), np.asarray(eps_b, np.float64)
    den = ea[p - 1] + eb[r - 1] - ea[q - 1] - eb[s - 1]
    return float(factor * np.sum(v * v / den))
