"""Seeded, counter-based synthetic inputs for the GCOO SpDM workloads.

Every value is a pure function of (seed, stream, index) through splitmix64, so
the same bytes come out of the NumPy path (host) and the torch path (device,
any backend) on any machine and any library version. The reference's own
generator (src/utils.cpp:5-19: unseeded rand(), values in [0,1]) is not used;
the workloads below follow the sparsity patterns and value distributions of
the benchmark configurations instead:

* ``bernoulli_dense``: each entry nonzero with probability p, values U(-1,1)
  (odd multiples of 2^-24, never exactly 0, so nnz equals the mask count).
* ``block_dense``: 16x16 blocks, each active with probability p, dense inside.
* ``zipf_coo``: per-row counts Zipf(alpha) capped and rescaled to an nnz
  target, distinct uniform columns per row, N(0,1) values.
* ``batched_shapes``: shapes/sparsities of the batched workload.
"""
from __future__ import annotations

import math

import numpy as np

_M64 = (1 << 64) - 1
_GOLD = 0x9E3779B97F4A7C15
_C1 = 0xBF58476D1CE4E5B9
_C2 = 0x94D049BB133111EB
_SK = 0xD1B54A32D192ED03


def _u64(x: int) -> np.uint64:
    return np.uint64(x & _M64)


def splitmix64_np(x: np.ndarray) -> np.ndarray:
    """splitmix64 finaliser on a uint64 array (wrapping arithmetic)."""
    with np.errstate(over="ignore"):
        z = x + _u64(_GOLD)
        z = (z ^ (z >> np.uint64(30))) * _u64(_C1)
        z = (z ^ (z >> np.uint64(27))) * _u64(_C2)
        return z ^ (z >> np.uint64(31))


def stream_key(seed: int, stream: int) -> int:
    x = np.array([(seed + stream * _SK) & _M64], dtype=np.uint64)
    return int(splitmix64_np(x)[0])


def hash_np(seed: int, stream: int, start: int, count: int) -> np.ndarray:
    key = stream_key(seed, stream)
    idx = np.arange(start, start + count, dtype=np.uint64)
    with np.errstate(over="ignore"):
        return splitmix64_np(idx + _u64(key))


def u01_from_hash(h: np.ndarray) -> np.ndarray:
    """53-bit uniform in [0,1) as float64."""
    return (h >> np.uint64(11)).astype(np.float64) * (1.0 / (1 << 53))


def pm1_from_hash(h: np.ndarray) -> np.ndarray:
    """U(-1,1) float32, odd multiples of 2^-24 (never 0, exact in FP32)."""
    u = (h >> np.uint64(40)).astype(np.int64)
    return ((2 * u + 1 - (1 << 24)).astype(np.float64) / float(1 << 24)).astype(np.float32)


def uniform_pm1(seed: int, stream: int, shape) -> np.ndarray:
    n = int(np.prod(shape))
    return pm1_from_hash(hash_np(seed, stream, 0, n)).reshape(shape)


def bernoulli_dense(seed: int, m: int, k: int, p: float, chunk_rows: int = 0) -> np.ndarray:
    """Dense m x k FP32 with i.i.d. Bernoulli(p) mask and U(-1,1) values."""
    out = np.empty((m, k), dtype=np.float32)
    thr = np.uint64(min(int(p * float(1 << 53)), 1 << 53))
    step = chunk_rows or max(1, (1 << 22) // max(k, 1))
    for r0 in range(0, m, step):
        r1 = min(m, r0 + step)
        n = (r1 - r0) * k
        hm = hash_np(seed, 1, r0 * k, n)
        hv = hash_np(seed, 2, r0 * k, n)
        keep = (hm >> np.uint64(11)) < thr
        out[r0:r1] = np.where(keep, pm1_from_hash(hv), np.float32(0)).reshape(r1 - r0, k)
    return out


def bernoulli_nnz(seed: int, m: int, k: int, p: float) -> int:
    """Nonzeros of bernoulli_dense(seed, m, k, p) (the mask alone; values are
    never zero)."""
    thr = np.uint64(min(int(p * float(1 << 53)), 1 << 53))
    step = max(1, (1 << 22) // max(k, 1))
    total = 0
    for r0 in range(0, m, step):
        r1 = min(m, r0 + step)
        total += int(np.count_nonzero((hash_np(seed, 1, r0 * k, (r1 - r0) * k) >> np.uint64(11)) < thr))
    return total


def dense_pm1(seed: int, stream: int, rows: int, cols: int) -> np.ndarray:
    out = np.empty((rows, cols), dtype=np.float32)
    step = max(1, (1 << 22) // max(cols, 1))
    for r0 in range(0, rows, step):
        r1 = min(rows, r0 + step)
        out[r0:r1] = pm1_from_hash(hash_np(seed, stream, r0 * cols, (r1 - r0) * cols)).reshape(r1 - r0, cols)
    return out


def block_dense(seed: int, m: int, k: int, p: float, bs: int = 16) -> np.ndarray:
    """Block-clustered mask: bs x bs blocks active with probability p, dense inside."""
    mb, kb = (m + bs - 1) // bs, (k + bs - 1) // bs
    thr = np.uint64(min(int(p * float(1 << 53)), 1 << 53))
    active = ((hash_np(seed, 3, 0, mb * kb) >> np.uint64(11)) < thr).reshape(mb, kb)
    mask = np.repeat(np.repeat(active, bs, axis=0), bs, axis=1)[:m, :k]
    vals = dense_pm1(seed, 2, m, k)
    return np.where(mask, vals, np.float32(0))


def normal_from_hash(h1: np.ndarray, h2: np.ndarray) -> np.ndarray:
    u1 = 1.0 - u01_from_hash(h1)  # (0, 1]
    u2 = u01_from_hash(h2)
    return (np.sqrt(-2.0 * np.log(u1)) * np.cos(2.0 * math.pi * u2)).astype(np.float32)


def zipf_coo(seed: int, m: int, k: int, nnz_target: int, alpha: float = 2.0, cap: int = 4096):
    """Irregular matrix as COO (rows, cols, vals), rows sorted, cols distinct per row.

    Row counts: Zipf(alpha) on 1..cap by inverse CDF, rescaled to nnz_target
    and capped at cap; the remainder is spread one per row in row order.
    """
    support = np.arange(1, cap + 1, dtype=np.float64)
    cdf = np.cumsum(support ** (-alpha))
    cdf /= cdf[-1]
    u = u01_from_hash(hash_np(seed, 10, 0, m))
    counts = np.searchsorted(cdf, u, side="right").astype(np.float64) + 1.0
    counts = np.minimum(np.floor(counts * (nnz_target / counts.sum())), cap).astype(np.int64)
    deficit = nnz_target - int(counts.sum())
    r = 0
    while deficit > 0:
        room = counts < cap
        idx = np.nonzero(room)[0][:deficit]
        counts[idx] += 1
        deficit -= len(idx)
        r += 1
        if r > 10000:
            break
    rows = np.repeat(np.arange(m, dtype=np.int64), counts)
    total = rows.size
    # distinct columns per row: draw, dedupe, redraw the collisions
    cols = (hash_np(seed, 11, 0, total) % np.uint64(k)).astype(np.int64)
    attempt = 0
    while True:
        key = rows * k + cols
        order = np.argsort(key, kind="stable")
        key_sorted = key[order]
        dup = np.zeros(total, dtype=bool)
        dup[order[1:]] = key_sorted[1:] == key_sorted[:-1]
        nd = int(dup.sum())
        if nd == 0:
            break
        attempt += 1
        cols[dup] = (hash_np(seed, 12 + attempt, 0, nd) % np.uint64(k)).astype(np.int64)
    order = np.lexsort((cols, rows))
    rows, cols = rows[order], cols[order]
    vals = normal_from_hash(hash_np(seed, 20, 0, total), hash_np(seed, 21, 0, total))
    vals[vals == 0] = np.float32(1e-3)
    return rows.astype(np.int64), cols.astype(np.int64), vals


def normal_dense(seed: int, stream: int, rows: int, cols: int) -> np.ndarray:
    n = rows * cols
    return normal_from_hash(hash_np(seed, stream, 0, n), hash_np(seed, stream + 1, 0, n)).reshape(rows, cols)


def batched_shapes(seed: int, count: int = 512):
    """(m, k, n, sparsity) per problem of the batched workload."""
    h = [hash_np(seed, 30 + i, 0, count) for i in range(4)]
    m = 256 + (h[0] % np.uint64(4096 - 256 + 1)).astype(np.int64)
    k = 256 + (h[1] % np.uint64(4096 - 256 + 1)).astype(np.int64)
    n = np.array([32, 64, 128], dtype=np.int64)[(h[2] % np.uint64(3)).astype(np.int64)]
    s = 0.9 + 0.099 * u01_from_hash(h[3])
    return [(int(m[i]), int(k[i]), int(n[i]), float(s[i])) for i in range(count)]


# ---- the same streams generated with torch (any device), for full-size inputs ----

def _s64(x: int) -> int:
    x &= _M64
    return x - (1 << 64) if x >= (1 << 63) else x


def _srl(z, s: int):
    """Logical right shift of int64 tensor bits."""
    return (z >> s) & ((1 << (64 - s)) - 1)


def splitmix64_torch(x):
    z = x + _s64(_GOLD)
    z = (z ^ _srl(z, 30)) * _s64(_C1)
    z = (z ^ _srl(z, 27)) * _s64(_C2)
    return z ^ _srl(z, 31)


def hash_torch(seed: int, stream: int, start: int, count: int, device):
    import torch
    key = _s64(stream_key(seed, stream))
    idx = torch.arange(start, start + count, dtype=torch.int64, device=device)
    return splitmix64_torch(idx + key)


def _pm1_torch(h):
    import torch
    u = _srl(h, 40)
    return ((2 * u + 1 - (1 << 24)).to(torch.float64) / float(1 << 24)).to(torch.float32)


def bernoulli_dense_torch(seed: int, m: int, k: int, p: float, device="cuda", chunk: int = 1 << 24):
    """Same values as bernoulli_dense, generated on `device`."""
    import torch
    out = torch.empty(m * k, dtype=torch.float32, device=device)
    thr = min(int(p * float(1 << 53)), 1 << 53)
    for s in range(0, m * k, chunk):
        n = min(chunk, m * k - s)
        keep = _srl(hash_torch(seed, 1, s, n, device), 11) < thr
        vals = _pm1_torch(hash_torch(seed, 2, s, n, device))
        out[s:s + n] = torch.where(keep, vals, torch.zeros_like(vals))
    return out.view(m, k)


def dense_pm1_torch(seed: int, stream: int, rows: int, cols: int, device="cuda", chunk: int = 1 << 24):
    import torch
    out = torch.empty(rows * cols, dtype=torch.float32, device=device)
    for s in range(0, rows * cols, chunk):
        n = min(chunk, rows * cols - s)
        out[s:s + n] = _pm1_torch(hash_torch(seed, stream, s, n, device))
    return out.view(rows, cols)


def block_dense_torch(seed: int, m: int, k: int, p: float, bs: int = 16, device="cuda"):
    """Same values as block_dense, generated on `device`."""
    import torch
    mb, kb = (m + bs - 1) // bs, (k + bs - 1) // bs
    thr = min(int(p * float(1 << 53)), 1 << 53)
    active = (_srl(hash_torch(seed, 3, 0, mb * kb, device), 11) < thr).view(mb, kb)
    mask = active.repeat_interleave(bs, 0).repeat_interleave(bs, 1)[:m, :k]
    vals = dense_pm1_torch(seed, 2, m, k, device)
    return torch.where(mask, vals, torch.zeros_like(vals))
