"""Seeded synthetic workloads with the shapes and distributions of the
benchmark configurations (no dataset is involved).

Every system s is drawn from its own generator ``default_rng([seed, s])``, so
any process can rebuild any subset of a workload without generating the rest
(the CPU baseline's worker processes rely on this).
"""

from __future__ import annotations

import dataclasses

import numpy as np


@dataclasses.dataclass
class RaggedSPD:
    """Ragged SPD batch: A_s = G Gᵀ/n + 1e-2·I (G i.i.d. N(0,1)), nrhs_s
    right-hand sides ~ N(0,1), packed row-major back to back."""

    seed: int
    n: list
    nrhs: list
    a: np.ndarray | None = None
    b: np.ndarray | None = None


def ragged_spd_sizes(seed: int, count: int = 4096, nmin: int = 16, nmax: int = 512,
                     kmin: int = 1, kmax: int = 8, sort_desc: bool = True):
    """Orders n ~ ⌊exp U(ln nmin, ln(nmax+1))⌋ (log-uniform on [nmin, nmax]) and
    nrhs ~ U{kmin..kmax}.  Sorted by decreasing n when sort_desc (the order
    the persistent kernel takes systems in; largest first balances it)."""
    rng = np.random.default_rng([seed, 0x5E5])
    n = np.floor(np.exp(rng.uniform(np.log(nmin), np.log(nmax + 1), size=count))).astype(int)
    n = np.clip(n, nmin, nmax)
    k = rng.integers(kmin, kmax + 1, size=count)
    if sort_desc:
        order = np.argsort(-n, kind="stable")
        n, k = n[order], k[order]
    return [int(v) for v in n], [int(v) for v in k]


def spd_system(seed: int, s: int, n: int, k: int):
    """System s of the workload: (A (n×n), B (k×n))."""
    rng = np.random.default_rng([seed, 1, s])
    g = rng.standard_normal((n, n))
    a = g @ g.T
    a /= n
    a[np.diag_indices(n)] += 1e-2
    b = rng.standard_normal((k, n))
    return a, b


def ragged_spd(seed: int = 0, count: int = 4096, **kw) -> RaggedSPD:
    """Build the whole packed workload (FP64 host arrays)."""
    n, k = ragged_spd_sizes(seed, count, **kw)
    ta = sum(v * v for v in n)
    tb = sum(v * r for v, r in zip(n, k))
    a = np.empty(ta, dtype=np.float64)
    b = np.empty(tb, dtype=np.float64)
    ao = bo = 0
    for s, (nv, kv) in enumerate(zip(n, k)):
        a_s, b_s = spd_system(seed, s, nv, kv)
        a[ao : ao + nv * nv] = a_s.reshape(-1)
        b[bo : bo + nv * kv] = b_s.reshape(-1)
        ao += nv * nv
        bo += nv * kv
    return RaggedSPD(seed, n, k, a, b)


def lu_batch(seed: int = 0, batch: int = 64, n: int = 128):
    """Equal-size LU batch: A = G/sqrt(n) + I, one b ~ N(0,1) per system."""
    rng = np.random.default_rng([seed, 2])
    a = rng.standard_normal((batch, n, n)) / np.sqrt(n) + np.eye(n)
    b = rng.standard_normal((batch, n))
    return a, b
