"""Seeded synthetic inputs standing in for the reference's datasets.

The reference runs on ``data/flickr.mtx`` and ``data/reddit.mtx``
(Makefile:22-30), which are not distributed with it.  These generators make
graphs of the same shape from a counter-based hash (murmur3 ``fmix32``) in
integer tensor ops, so a graph is identical whether it is generated on the
CPU or on a GPU.  Floating-point features are drawn from the same hash;
their last bits may differ between devices (log/cos), which only matters if
a caller generates them on two devices and compares.

Workloads (sizes as stated for the evaluation):
  * ``uniform_rows``: n x n, exactly k distinct uniformly random columns per
    row, values U[-1, 1]  (4096 x 4096, k = 16).
  * ``chung_lu``: undirected Chung-Lu graph whose expected degrees follow a
    truncated power law P(d) ~ d^-gamma on [dmin, dmax], self-loops removed,
    symmetrised and deduplicated, values 1.0.  ``flickr_like`` (89,250
    nodes, gamma 2.0, ~0.9M directed edges) and ``reddit_like`` (232,965
    nodes, gamma 1.8, degrees capped at 20,000, ~114.6M directed edges).
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import torch

_M32 = 0xFFFFFFFF


def _mul32(h: torch.Tensor, c: int) -> torch.Tensor:
    """(h * c) mod 2^32 for 0 <= h < 2^32 without int64 overflow."""
    lo = (h & 0xFFFF) * c
    hi = ((h >> 16) * c) & 0xFFFF
    return (lo + (hi << 16)) & _M32


def _fmix32(h: torch.Tensor) -> torch.Tensor:
    h = h ^ (h >> 16)
    h = _mul32(h, 0x85EBCA6B)
    h = h ^ (h >> 13)
    h = _mul32(h, 0xC2B2AE35)
    return h ^ (h >> 16)


def _fmix32_int(h: int) -> int:
    h ^= h >> 16
    h = (h * 0x85EBCA6B) & _M32
    h ^= h >> 13
    h = (h * 0xC2B2AE35) & _M32
    return h ^ (h >> 16)


def hash32(seed: int, stream: int, idx: torch.Tensor) -> torch.Tensor:
    """32-bit hash of (seed, stream, idx) for an int64 index tensor."""
    k = _fmix32_int((seed * 0x9E3779B1 + stream * 0x85EBCA77 + 0x165667B1) & _M32)
    k2 = _fmix32_int(k ^ 0x27D4EB2F)
    h = _fmix32((idx & _M32) ^ k)
    return _fmix32(h ^ ((idx >> 32) & _M32) ^ k2)


def uniform01(seed: int, stream: int, idx: torch.Tensor) -> torch.Tensor:
    """float64 uniform in [0, 1) with 53 random bits."""
    a = hash32(seed, 2 * stream, idx) >> 5          # 27 bits
    b = hash32(seed, 2 * stream + 1, idx) >> 6      # 26 bits
    return (a.double() * 67108864.0 + b.double()) * (1.0 / 9007199254740992.0)


def normal(seed: int, stream: int, shape: tuple[int, ...], device="cpu",
           dtype=torch.float32) -> torch.Tensor:
    """N(0, 1) samples by Box-Muller from the hash stream."""
    n = math.prod(shape)
    idx = torch.arange(n, dtype=torch.int64, device=device)
    u1 = uniform01(seed, 2 * stream, idx)
    u2 = uniform01(seed, 2 * stream + 1, idx)
    r = torch.sqrt(-2.0 * torch.log1p(-u1))
    z = r * torch.cos(2.0 * math.pi * u2)
    return z.to(dtype).reshape(shape)


@dataclass
class Graph:
    """Host- or device-resident CSR (int32 rowptr/colind, float32 vals)."""

    rowptr: torch.Tensor
    colind: torch.Tensor
    vals: torch.Tensor
    nrows: int
    ncols: int
    name: str = ""

    @property
    def nnz(self) -> int:
        return int(self.colind.numel())

    def to(self, device) -> "Graph":
        return Graph(self.rowptr.to(device), self.colind.to(device), self.vals.to(device),
                     self.nrows, self.ncols, self.name)

    def degrees(self) -> torch.Tensor:
        return (self.rowptr[1:] - self.rowptr[:-1]).to(torch.int64)


def _csr_from_sorted_keys(keys: torch.Tensor, n: int, m: int) -> tuple[torch.Tensor, torch.Tensor]:
    rows = keys // m
    cols = keys - rows * m
    counts = torch.bincount(rows, minlength=n)
    rowptr = torch.zeros(n + 1, dtype=torch.int64, device=keys.device)
    rowptr[1:] = torch.cumsum(counts, 0)
    return rowptr.to(torch.int32), cols.to(torch.int32)


def uniform_rows(n: int = 4096, k: int = 16, seed: int = 0x5EED + 1, device="cpu",
                 chunk_rows: int = 1024) -> Graph:
    """n x n CSR with exactly k distinct uniform columns per row, vals U[-1,1]."""
    if k > n:
        raise ValueError("k > n")
    cols_all = []
    for r0 in range(0, n, chunk_rows):
        r1 = min(n, r0 + chunk_rows)
        idx = (torch.arange(r0, r1, dtype=torch.int64, device=device)[:, None] * n
               + torch.arange(n, dtype=torch.int64, device=device)[None, :])
        h = hash32(seed, 0, idx)
        # k smallest hash values per row -> k distinct columns (ties by column)
        keyed = h * n + torch.arange(n, dtype=torch.int64, device=device)[None, :]
        sel = torch.topk(keyed, k, dim=1, largest=False).values % n
        cols_all.append(torch.sort(sel, dim=1).values)
    cols = torch.cat(cols_all, 0).reshape(-1)
    rowptr = torch.arange(0, n * k + 1, k, dtype=torch.int32, device=device)
    vals = (2.0 * uniform01(seed, 1, torch.arange(n * k, dtype=torch.int64, device=device)) - 1.0)
    return Graph(rowptr, cols.to(torch.int32), vals.to(torch.float32), n, n, f"uniform{n}x{k}")


def power_law_weights(n: int, gamma: float, dmin: float, dmax: float, device="cpu") -> torch.Tensor:
    """Expected degrees at quantiles (i + 0.5) / n of a power law on [dmin, dmax]."""
    q = (torch.arange(n, dtype=torch.float64, device=device) + 0.5) / n
    a = 1.0 - gamma
    lo, hi = dmin ** a, dmax ** a
    return (lo - q * (lo - hi)) ** (1.0 / a)


def chung_lu(n: int, gamma: float, dmin: float, dmax: float, seed: int, device="cpu",
             name: str = "chung_lu") -> Graph:
    """Undirected Chung-Lu graph, no self-loops, deduplicated, values 1.0.

    Node ids are a hash permutation of the degree ranks, so hubs are spread
    over the id range as in real graphs.
    """
    # Weights in 2^-20 fixed point, computed on the CPU, so the cumulative
    # sums (and hence every sampled endpoint) are exact integers on any device.
    w = power_law_weights(n, gamma, dmin, dmax, "cpu")
    ar = torch.arange(n, dtype=torch.int64)
    perm = torch.argsort(hash32(seed, 7, ar) * n + ar)
    wq = torch.round(w[perm] * 1048576.0).to(torch.int64).to(device)
    cum = torch.cumsum(wq, 0)
    total = int(cum[-1])
    m = int(round(total / 2097152.0))
    out_keys = []
    step = 1 << 24
    for s0 in range(0, m, step):
        idx = torch.arange(s0, min(m, s0 + step), dtype=torch.int64, device=device)
        pu = torch.floor(uniform01(seed, 1, idx) * float(total)).to(torch.int64)
        pv = torch.floor(uniform01(seed, 2, idx) * float(total)).to(torch.int64)
        u = torch.searchsorted(cum, pu, right=True).clamp_(max=n - 1)
        v = torch.searchsorted(cum, pv, right=True).clamp_(max=n - 1)
        keep = u != v
        u, v = u[keep], v[keep]
        out_keys.append(torch.unique(torch.cat([u * n + v, v * n + u])))
    keys = torch.unique(torch.cat(out_keys)) if len(out_keys) > 1 else out_keys[0]
    rowptr, colind = _csr_from_sorted_keys(keys, n, n)
    vals = torch.ones(colind.numel(), dtype=torch.float32, device=device)
    return Graph(rowptr, colind, vals, n, n, name)


def flickr_like(seed: int = 0x5EED + 2, device="cpu") -> Graph:
    """89,250 nodes, power-law exponent 2.0, about 0.9M directed edges."""
    return chung_lu(89_250, 2.0, 1.33, 5_000.0, seed, device, "flickr_like")


def reddit_like(seed: int = 0x5EED + 4, device="cpu") -> Graph:
    """232,965 nodes, exponent 1.8, degrees capped at 20,000, ~114.6M edges."""
    return chung_lu(232_965, 1.8, 59.9, 20_000.0, seed, device, "reddit_like")


def gcn_normalize(g: Graph) -> Graph:
    """Values D^-1/2 A D^-1/2 (degree = row count), computed in FP64 and
    stored FP32, on the graph's own device."""
    deg = g.degrees().double()
    dinv = torch.where(deg > 0, deg.rsqrt(), torch.zeros_like(deg))
    rows = torch.repeat_interleave(torch.arange(g.nrows, device=g.rowptr.device),
                                   g.degrees())
    v = dinv[rows] * g.vals.double() * dinv[g.colind.long()]
    return Graph(g.rowptr, g.colind, v.to(torch.float32), g.nrows, g.ncols, g.name + "_norm")


def induced_subgraph(g: Graph, nodes: torch.Tensor) -> Graph:
    """Subgraph induced by `nodes` (relabelled 0..k-1 in the given order)."""
    g = g.to("cpu")
    nodes = nodes.to("cpu").long()
    k = nodes.numel()
    remap = torch.full((g.nrows,), -1, dtype=torch.int64)
    remap[nodes] = torch.arange(k)
    rows = torch.repeat_interleave(torch.arange(g.nrows), g.degrees())
    cols = g.colind.long()
    keep = (remap[rows] >= 0) & (remap[cols] >= 0)
    r, c, v = remap[rows[keep]], remap[cols[keep]], g.vals[keep]
    order = torch.argsort(r * k + c)
    r, c, v = r[order], c[order], v[order]
    counts = torch.bincount(r, minlength=k)
    rowptr = torch.zeros(k + 1, dtype=torch.int64)
    rowptr[1:] = torch.cumsum(counts, 0)
    return Graph(rowptr.to(torch.int32), c.to(torch.int32), v.to(torch.float32), k, k,
                 g.name + f"_sub{k}")
