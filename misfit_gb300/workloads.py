"""Synthetic inputs in MISFIT's own formats.

* ``.egr`` binary CSR (int32 or int64-sentinel ``nindex``), read and written
  exactly as the reference describes it (README "File formats";
  core/FlashGraph.h:108-169 reads it, tools/efficient_converter.py writes the
  int64 form only).
* Graph families of the benchmark configurations: Erdos-Renyi G(n, m),
  R-MAT, and 2-D random geometric graphs.  All are undirected, stored with
  both directions, without self-loops or duplicates, rows sorted ascending.
* Update streams of toggles: deletes of existing edges and inserts of
  non-adjacent pairs, drawn against the nominal graph as it evolves.
* The initial-MIS and batch-folder text formats (one 1-indexed id per line;
  ``k.mtx`` files of ``u v`` lines, 1-indexed).

Everything is numpy and seeded, so the same arguments give the same bytes on
every machine.
"""
import os
import struct

import numpy as np

__all__ = [
    "read_egr", "write_egr", "csr_from_pairs", "er_graph", "rmat_graph", "rmat_graph_torch", "rgg_graph",
    "rgg_graph_torch", "ToggleStream", "DeviceToggles", "write_batch_file", "write_batch_folder", "read_batch_file",
    "write_mis_file", "read_mis_file", "undirected_pairs",
]


def read_egr(path):
    """Return (n, nindex int64[n+1], nlist int32[E], wide)."""
    with open(path, "rb") as f:
        n, e32 = struct.unpack("<ii", f.read(8))
        if e32 == -1:
            (e,) = struct.unpack("<Q", f.read(8))
            nindex = np.fromfile(f, dtype="<i8", count=n + 1)
            wide = True
        else:
            e = e32
            nindex = np.fromfile(f, dtype="<i4", count=n + 1).astype(np.int64)
            wide = False
        nlist = np.fromfile(f, dtype="<i4", count=e)
    if nindex.size != n + 1 or nlist.size != e:
        raise ValueError("truncated .egr file: %s" % path)
    return n, nindex, nlist, wide


def write_egr(path, n, nindex, nlist, wide=None):
    """Write a .egr file.  ``wide`` None picks int32 when the entry count fits."""
    nindex = np.asarray(nindex, dtype=np.int64)
    nlist = np.asarray(nlist, dtype=np.int32)
    e = int(nlist.size)
    if wide is None:
        wide = e > 0x7FFFFFFF
    tmp = path + ".tmp"
    with open(tmp, "wb") as f:
        if wide:
            f.write(struct.pack("<iiQ", n, -1, e))
            f.write(nindex.astype("<i8").tobytes())
        else:
            if e > 0x7FFFFFFF:
                raise ValueError("int32 layout cannot hold %d entries" % e)
            f.write(struct.pack("<ii", n, e))
            f.write(nindex.astype("<i4").tobytes())
        (nlist if nlist.dtype == np.dtype("<i4") else nlist.astype("<i4")).tofile(f)
    os.replace(tmp, path)


def csr_from_pairs(n, u, v):
    """Symmetric CSR with sorted rows from undirected pairs (self-loops and
    duplicates removed)."""
    u = np.asarray(u, dtype=np.int64)
    v = np.asarray(v, dtype=np.int64)
    keep = u != v
    u, v = u[keep], v[keep]
    key = np.concatenate([u * n + v, v * n + u])
    key = np.unique(key)
    src = key // n
    dst = (key % n).astype(np.int32)
    deg = np.bincount(src, minlength=n).astype(np.int64)
    nindex = np.zeros(n + 1, dtype=np.int64)
    np.cumsum(deg, out=nindex[1:])
    return nindex, dst


def undirected_pairs(n, nindex, nlist):
    """Unique undirected pairs (lo, hi) of a symmetric CSR, sorted by key."""
    deg = np.diff(nindex)
    src = np.repeat(np.arange(n, dtype=np.int64), deg)
    dst = nlist.astype(np.int64)
    sel = src < dst
    return src[sel], dst[sel]


def er_graph(n, avg_degree, seed):
    """G(n, m) with m = n*avg_degree/2 distinct undirected edges."""
    rng = np.random.default_rng(seed)
    m = int(round(n * avg_degree / 2))
    keys = np.empty(0, dtype=np.int64)
    while keys.size < m:
        need = m - keys.size
        a = rng.integers(0, n, size=2 * need + 16)
        b = rng.integers(0, n, size=2 * need + 16)
        ok = a != b
        lo = np.minimum(a[ok], b[ok])
        hi = np.maximum(a[ok], b[ok])
        new = lo * n + hi
        keys = np.unique(np.concatenate([keys, new]))
        if keys.size > m:
            # keep a seeded random subset of exactly m keys
            keys = np.sort(rng.choice(keys, size=m, replace=False))
    return csr_from_pairs(n, keys // n, keys % n)


def rmat_graph(scale, edge_factor, seed, abcd=(0.57, 0.19, 0.19, 0.05), chunk=1 << 24):
    """R-MAT with 2**scale vertices and edge_factor * 2**scale samples,
    symmetrised and de-duplicated."""
    a, b, c, _ = abcd
    n = 1 << scale
    total = n * edge_factor
    rng = np.random.default_rng(seed)
    keys = []
    done = 0
    while done < total:
        cnt = min(chunk, total - done)
        u = np.zeros(cnt, dtype=np.int64)
        v = np.zeros(cnt, dtype=np.int64)
        for lvl in range(scale):
            r = rng.random(cnt, dtype=np.float32)
            ubit = r >= (a + b)
            vbit = ((r >= a) & (r < a + b)) | (r >= (a + b + c))
            u |= ubit.astype(np.int64) << lvl
            v |= vbit.astype(np.int64) << lvl
        keep = u != v
        lo = np.minimum(u[keep], v[keep])
        hi = np.maximum(u[keep], v[keep])
        keys.append(np.unique(lo * n + hi))
        done += cnt
    key = np.unique(np.concatenate(keys))
    return n, csr_from_pairs(n, key // n, key % n)


def rgg_graph(n, mean_degree, seed):
    """2-D random geometric graph in the unit square with the radius set for
    the requested mean degree (with a first-order boundary correction)."""
    rng = np.random.default_rng(seed)
    pts = rng.random((n, 2))
    # expected degree with boundary loss ~ n*pi*r^2*(1 - 8r/(3pi))
    r = np.sqrt(mean_degree / (n * np.pi))
    for _ in range(3):
        r = np.sqrt(mean_degree / (n * np.pi * max(1e-9, 1 - 8 * r / (3 * np.pi))))
    cells = max(1, int(1.0 / r))
    cx = np.minimum((pts[:, 0] * cells).astype(np.int64), cells - 1)
    cy = np.minimum((pts[:, 1] * cells).astype(np.int64), cells - 1)
    cell = cx * cells + cy
    order = np.argsort(cell, kind="stable")
    cell_sorted = cell[order]
    starts = np.searchsorted(cell_sorted, np.arange(cells * cells + 1))
    us, vs = [], []
    r2 = r * r
    for dx in (-1, 0, 1):
        for dy in (-1, 0, 1):
            ncx = cx + dx
            ncy = cy + dy
            ok = (ncx >= 0) & (ncx < cells) & (ncy >= 0) & (ncy < cells)
            idx = np.nonzero(ok)[0]
            nc = ncx[idx] * cells + ncy[idx]
            lo = starts[nc]
            hi = starts[nc + 1]
            cnt = hi - lo
            rep = np.repeat(idx, cnt)
            off = np.arange(cnt.sum()) - np.repeat(np.cumsum(cnt) - cnt, cnt)
            cand = order[np.repeat(lo, cnt) + off]
            d = pts[rep] - pts[cand]
            close = (d * d).sum(axis=1) <= r2
            sel = close & (rep < cand)
            us.append(rep[sel])
            vs.append(cand[sel])
    return csr_from_pairs(n, np.concatenate(us), np.concatenate(vs))


class ToggleStream:
    """Batches of toggles drawn against the nominal graph as it evolves.

    Each batch holds ``batch_size`` lines: ``round(batch_size*delete_frac)``
    deletes of existing edges (uniform over the current edges) and the rest
    inserts of non-adjacent pairs, shuffled, each line in a random direction.
    ``endpoints`` picks how insert endpoints are drawn: ``uniform``,
    ``preferential`` (probability proportional to current degree) or
    ``low_degree`` (proportional to 1/max(degree, 1)); for the two weighted
    modes a delete keeps a sampled edge with probability proportional to the
    product of its endpoint weights.  After each batch the nominal graph
    applies the toggles, so later batches may delete edges inserted earlier.

    The base edge set stays a sorted array with an alive mask; inserted pairs
    that are not base edges live in a small sorted side array, so one batch
    costs O(batch * log E) whatever the graph size.
    """

    def __init__(self, n, nindex, nlist, seed):
        self.n = int(n)
        lo, hi = undirected_pairs(self.n, np.asarray(nindex, np.int64), np.asarray(nlist))
        self.base = lo * self.n + hi          # ascending: rows sorted, sources ascending
        if self.base.size > 1 and not np.all(self.base[1:] > self.base[:-1]):
            self.base = np.unique(self.base)
        self.alive = np.ones(self.base.size, dtype=bool)
        self.extra = np.empty(0, dtype=np.int64)
        self.rng = np.random.default_rng(seed)
        self.deg = np.diff(np.asarray(nindex, dtype=np.int64)).astype(np.float64)

    @property
    def num_edges(self):
        return int(self.alive.sum()) + int(self.extra.size)

    def _find(self, arr, keys):
        if arr.size == 0:
            return np.zeros(keys.shape, np.int64), np.zeros(keys.shape, bool)
        pos = np.minimum(np.searchsorted(arr, keys), arr.size - 1)
        return pos, arr[pos] == keys

    def _adjacent(self, keys):
        pos, hit = self._find(self.base, keys)
        a = hit & self.alive[pos]
        _, e = self._find(self.extra, keys)
        return a | e

    def _weights(self, mode):
        if mode == "preferential":
            return self.deg + 1e-12
        if mode == "low_degree":
            return 1.0 / np.maximum(self.deg, 1.0)
        raise ValueError(mode)

    def _vertices(self, mode, size):
        if mode == "uniform":
            return self.rng.integers(0, self.n, size=size)
        cdf = np.cumsum(self._weights(mode))
        cdf /= cdf[-1]
        return np.minimum(np.searchsorted(cdf, self.rng.random(size)), self.n - 1)

    def _sample_edges(self, count, mode):
        total = self.base.size + self.extra.size
        got = np.empty(0, dtype=np.int64)
        if count <= 0 or total == 0:
            return got
        w = None if mode == "uniform" else self._weights(mode)
        wmax = None if w is None else float(w.max()) ** 2
        while got.size < count:
            r = self.rng.integers(0, total, size=4 * (count - got.size) + 64)
            inb = r < self.base.size
            rb = r[inb]
            k = np.concatenate([self.base[rb[self.alive[rb]]], self.extra[r[~inb] - self.base.size]])
            if w is not None:
                a, b = k // self.n, k % self.n
                k = k[self.rng.random(k.size) * wmax < w[a] * w[b]]
            got = np.unique(np.concatenate([got, k]))
            if got.size > count:
                got = self.rng.permutation(got)[:count]
        return got

    def next_batch(self, batch_size, delete_frac=0.5, endpoints="uniform", with_flags=False):
        """(u, v), or (u, v, ins) with ins = 1 for inserts and 0 for deletes
        when with_flags (the flags against the nominal graph, which is what a
        serving client sends)."""
        n = self.n
        nd = min(int(round(batch_size * delete_frac)), self.num_edges)
        ni = batch_size - nd
        dkeys = self._sample_edges(nd, endpoints)
        ikeys = np.empty(0, dtype=np.int64)
        while ikeys.size < ni:
            need = ni - ikeys.size
            a = self._vertices(endpoints, 2 * need + 16)
            b = self._vertices(endpoints, 2 * need + 16)
            ok = a != b
            lo = np.minimum(a[ok], b[ok])
            hi = np.maximum(a[ok], b[ok])
            k = lo * n + hi
            k = k[~self._adjacent(k)]
            ikeys = np.unique(np.concatenate([ikeys, k]))
            if ikeys.size > ni:
                ikeys = self.rng.permutation(ikeys)[:ni]
        keys = np.concatenate([dkeys, ikeys])
        is_ins = np.concatenate([np.zeros(dkeys.size, np.uint8), np.ones(ikeys.size, np.uint8)])
        perm = self.rng.permutation(keys.size)
        keys = keys[perm]
        is_ins = is_ins[perm]
        lo = keys // n
        hi = keys % n
        flip = self.rng.random(keys.size) < 0.5
        u = np.where(flip, hi, lo).astype(np.int32)
        v = np.where(flip, lo, hi).astype(np.int32)
        # nominal graph update
        pos, inb = self._find(self.base, dkeys)
        self.alive[pos[inb]] = False
        if (~inb).any():
            self.extra = np.setdiff1d(self.extra, dkeys[~inb], assume_unique=True)
        pos, inb = self._find(self.base, ikeys)
        self.alive[pos[inb]] = True
        if (~inb).any():
            self.extra = np.union1d(self.extra, ikeys[~inb])
        for keyset, sign in ((dkeys, -1.0), (ikeys, 1.0)):
            np.add.at(self.deg, keyset // n, sign)
            np.add.at(self.deg, keyset % n, sign)
        if with_flags:
            return u, v, is_ins
        return u, v


def rmat_graph_torch(scale, edge_factor, seed, device="cuda", abcd=(0.57, 0.19, 0.19, 0.05)):
    """R-MAT as rmat_graph, generated on a CUDA device with torch (Philox
    stream seeded by ``seed``); returns host numpy arrays (n, (nindex, nlist)).
    Used for the large benchmark graphs, which numpy builds too slowly.  The
    keys are de-duplicated and sorted per range of source vertices (at most
    2^30 keys per sort), so that graphs beyond 2^31 directed entries build
    without one giant sort; the result is the same as one global sort."""
    import torch

    a, b, c, _ = abcd
    n = 1 << scale
    total = n * edge_factor
    gen = torch.Generator(device=device)
    gen.manual_seed(seed)
    nbuck = max(1, -(-2 * total // (1 << 30)))
    bounds = [(n * k) // nbuck for k in range(nbuck + 1)]
    buckets = [[] for _ in range(nbuck)]
    chunk = 1 << 25
    done = 0
    while done < total:
        cnt = min(chunk, total - done)
        u = torch.zeros(cnt, dtype=torch.int64, device=device)
        v = torch.zeros(cnt, dtype=torch.int64, device=device)
        for lvl in range(scale):
            r = torch.rand(cnt, generator=gen, device=device)
            u |= (r >= (a + b)).to(torch.int64) << lvl
            v |= (((r >= a) & (r < a + b)) | (r >= (a + b + c))).to(torch.int64) << lvl
        keep = u != v
        lo = torch.minimum(u[keep], v[keep])
        hi = torch.maximum(u[keep], v[keep])
        key = torch.unique(lo * n + hi)
        for k in range(nbuck):
            sel = key[(key >= bounds[k] * n) & (key < bounds[k + 1] * n)]
            if sel.numel():
                buckets[k].append(sel)
        done += cnt
    # unique undirected keys, lo < hi, per bucket of lo
    ukeys = []
    for k in range(nbuck):
        ukeys.append(torch.unique(torch.cat(buckets[k])) if buckets[k] else
                     torch.zeros(0, dtype=torch.int64, device=device))
        buckets[k] = None
    # both directions, sorted per bucket of the source vertex
    deg = torch.zeros(n, dtype=torch.int64, device=device)
    for uk in ukeys:
        deg += torch.bincount(uk // n, minlength=n) + torch.bincount(uk % n, minlength=n)
    nindex = torch.zeros(n + 1, dtype=torch.int64, device=device)
    nindex[1:] = torch.cumsum(deg, 0)
    nlist = np.empty(int(nindex[-1].item()), dtype=np.int32)
    for k in range(nbuck):
        lo_b, hi_b = bounds[k] * n, bounds[k + 1] * n
        parts = [ukeys[k]]                                 # (lo, hi) with lo in the bucket
        for uk in ukeys:                                   # (hi, lo) with hi in the bucket
            h = uk % n
            m = (h >= bounds[k]) & (h < bounds[k + 1])
            if m.any():
                parts.append(h[m] * n + uk[m] // n)
        both = torch.sort(torch.cat(parts)).values
        del parts
        if both.numel():
            assert int(both[0].item()) >= lo_b and int(both[-1].item()) < hi_b
            start = int(nindex[bounds[k]].item())
            nlist[start:start + both.numel()] = (both % n).to(torch.int32).cpu().numpy()
        del both
    del ukeys
    return n, (nindex.cpu().numpy(), nlist)


def rgg_graph_torch(n, mean_degree, seed, device="cuda"):
    """2-D random geometric graph as rgg_graph (points uniform in the unit
    square, radius set for the mean degree with the same boundary
    correction), generated on a CUDA device with torch from its own seeded
    stream: the same distribution as rgg_graph, not the same graph.  Returns
    host numpy arrays (nindex int64, nlist int32), rows sorted ascending."""
    import torch

    gen = torch.Generator(device=device)
    gen.manual_seed(seed)
    pts = torch.rand((n, 2), generator=gen, device=device, dtype=torch.float64)
    r = np.sqrt(mean_degree / (n * np.pi))
    for _ in range(3):
        r = np.sqrt(mean_degree / (n * np.pi * max(1e-9, 1 - 8 * r / (3 * np.pi))))
    cells = max(1, int(1.0 / r))
    cx = (pts[:, 0] * cells).long().clamp_(max=cells - 1)
    cy = (pts[:, 1] * cells).long().clamp_(max=cells - 1)
    cell = cx * cells + cy
    order = torch.argsort(cell)
    starts = torch.searchsorted(cell[order], torch.arange(cells * cells + 1, device=device))
    r2 = r * r
    us, vs = [], []
    for dx in (-1, 0, 1):
        for dy in (-1, 0, 1):
            ncx, ncy = cx + dx, cy + dy
            idx = ((ncx >= 0) & (ncx < cells) & (ncy >= 0) & (ncy < cells)).nonzero().squeeze(1)
            nc = ncx[idx] * cells + ncy[idx]
            lo = starts[nc]
            cnt = starts[nc + 1] - lo
            tot = int(cnt.sum().item())
            if tot == 0:
                continue
            rep = torch.repeat_interleave(idx, cnt)
            off = torch.arange(tot, device=device) - torch.repeat_interleave(torch.cumsum(cnt, 0) - cnt, cnt)
            cand = order[torch.repeat_interleave(lo, cnt) + off]
            d = pts[rep] - pts[cand]
            sel = ((d * d).sum(dim=1) <= r2) & (rep < cand)
            us.append(rep[sel])
            vs.append(cand[sel])
    u = torch.cat(us) if us else torch.zeros(0, dtype=torch.int64, device=device)
    v = torch.cat(vs) if vs else torch.zeros(0, dtype=torch.int64, device=device)
    both = torch.sort(torch.cat([u * n + v, v * n + u])).values
    src = both // n
    nindex = torch.zeros(n + 1, dtype=torch.int64, device=device)
    nindex[1:] = torch.cumsum(torch.bincount(src, minlength=n), 0)
    return nindex.cpu().numpy(), (both % n).to(torch.int32).cpu().numpy()


class DeviceToggles:
    """Batches of toggles drawn on a CUDA device against a graph's base CSR,
    for graphs too large (or too many) for ToggleStream's host arrays.

    A batch holds ``round(size*delete_frac)`` deletes of distinct base edges
    and the rest inserts of distinct non-adjacent pairs (u != v), shuffled,
    each line in a random direction.  ``endpoints``:
      * ``uniform``: deletes uniform over the edges, insert endpoints uniform;
      * ``preferential``: endpoints proportional to degree -- deletes uniform
        over the edges (each endpoint of a uniform edge is degree-
        proportional), insert endpoints drawn independently by degree;
      * ``low_degree``: proportional to 1/max(degree, 1) -- a delete keeps a
        uniform edge with probability w(u)*w(v), insert endpoints by weight.
    Draws are against the base graph: a graph that takes many batches sees
    deletes of edges an earlier batch may have deleted already (no-ops for
    the overlay), as a client working from a stale copy would send them.
    ``adjacent(a, b)`` (torch int64 tensors -> bool tensor) tests base
    adjacency; by default a sorted key array of the base entries is built
    on the device."""

    def __init__(self, nindex, nlist, seed, device="cuda", adjacent=None):
        import torch

        self.torch = torch
        self.dev = device
        self.nindex = torch.as_tensor(np.asarray(nindex, np.int64), device=device)
        self.n = int(self.nindex.numel() - 1)
        self.nlist = torch.as_tensor(np.asarray(nlist, np.int32), device=device)
        self.E = int(self.nlist.numel())
        self.deg = (self.nindex[1:] - self.nindex[:-1]).to(torch.float64)
        self.gen = torch.Generator(device=device)
        self.gen.manual_seed(seed)
        if adjacent is None:
            src = torch.repeat_interleave(torch.arange(self.n, device=device),
                                          (self.nindex[1:] - self.nindex[:-1]))
            self.keys = src * self.n + self.nlist.to(torch.int64)   # ascending: sorted rows
            adjacent = self._adjacent_keys
        self.adjacent = adjacent
        self._cdf = {}

    def _adjacent_keys(self, a, b):
        torch = self.torch
        k = a * self.n + b
        if self.E == 0:
            return torch.zeros(k.shape, dtype=torch.bool, device=self.dev)
        pos = torch.searchsorted(self.keys, k).clamp_(max=self.E - 1)
        return self.keys[pos] == k

    def _weights(self, mode):
        if mode == "preferential":
            return self.deg + 1e-12
        return 1.0 / self.deg.clamp(min=1.0)

    def _vertices(self, mode, size):
        torch = self.torch
        if mode == "uniform":
            return torch.randint(0, self.n, (size,), generator=self.gen, device=self.dev)
        if mode not in self._cdf:
            self._cdf[mode] = torch.cumsum(self._weights(mode), 0)
        cdf = self._cdf[mode]
        x = torch.rand(size, generator=self.gen, device=self.dev, dtype=torch.float64) * cdf[-1]
        return torch.searchsorted(cdf, x).clamp_(max=self.n - 1)

    def _edges(self, mode, count):
        torch = self.torch
        got = torch.zeros(0, dtype=torch.int64, device=self.dev)
        if count <= 0 or self.E == 0:
            return got
        w = None if mode in ("uniform", "preferential") else self._weights(mode)
        while got.numel() < count:
            need = count - got.numel()
            draws = 4 * need + 64 if w is None else 64 * need + 1024
            pos = torch.randint(0, self.E, (draws,), generator=self.gen, device=self.dev)
            a = torch.searchsorted(self.nindex, pos, right=True) - 1
            b = self.nlist[pos].to(torch.int64)
            if w is not None:
                keep = torch.rand(draws, generator=self.gen, device=self.dev, dtype=torch.float64) < w[a] * w[b]
                a, b = a[keep], b[keep]
            k = torch.minimum(a, b) * self.n + torch.maximum(a, b)
            got = torch.unique(torch.cat([got, k]))
            if got.numel() > count:
                got = got[torch.randperm(got.numel(), generator=self.gen, device=self.dev)[:count]]
        return got

    def next_batch(self, size, delete_frac=0.5, endpoints="uniform"):
        """(u, v, ins) host numpy arrays (int32, int32, uint8); ins is 1 for
        an insert (non-adjacent in the base graph) and 0 for a delete."""
        torch = self.torch
        n = self.n
        nd = min(int(round(size * delete_frac)), self.E // 2)
        ni = size - nd
        dkeys = self._edges(endpoints, nd)
        ikeys = torch.zeros(0, dtype=torch.int64, device=self.dev)
        tries = 0
        while ikeys.numel() < ni and tries < 64:
            tries += 1
            need = ni - ikeys.numel()
            a = self._vertices(endpoints, 2 * need + 16)
            b = self._vertices(endpoints, 2 * need + 16)
            ok = a != b
            lo, hi = torch.minimum(a[ok], b[ok]), torch.maximum(a[ok], b[ok])
            keep = ~self.adjacent(lo, hi)
            ikeys = torch.unique(torch.cat([ikeys, lo[keep] * n + hi[keep]]))
            if ikeys.numel() > ni:
                ikeys = ikeys[torch.randperm(ikeys.numel(), generator=self.gen, device=self.dev)[:ni]]
        keys = torch.cat([dkeys, ikeys])
        ins = torch.cat([torch.zeros(dkeys.numel(), dtype=torch.uint8, device=self.dev),
                         torch.ones(ikeys.numel(), dtype=torch.uint8, device=self.dev)])
        perm = torch.randperm(keys.numel(), generator=self.gen, device=self.dev)
        keys, ins = keys[perm], ins[perm]
        lo, hi = keys // n, keys % n
        flip = torch.rand(keys.numel(), generator=self.gen, device=self.dev) < 0.5
        u = torch.where(flip, hi, lo).to(torch.int32)
        v = torch.where(flip, lo, hi).to(torch.int32)
        return u.cpu().numpy(), v.cpu().numpy(), ins.cpu().numpy()


def write_batch_file(path, u, v):
    """``u v`` lines, 1-indexed."""
    arr = np.stack([np.asarray(u, np.int64) + 1, np.asarray(v, np.int64) + 1], axis=1)
    with open(path, "w") as f:
        if arr.size:
            f.write("\n".join("%d %d" % (a, b) for a, b in arr))
            f.write("\n")


def write_batch_folder(folder, batches):
    os.makedirs(folder, exist_ok=True)
    for i, (u, v) in enumerate(batches):
        write_batch_file(os.path.join(folder, "%d.mtx" % (i + 1)), u, v)


def read_batch_file(path):
    """0-indexed (u, v) of every line that starts with two integers."""
    us, vs = [], []
    with open(path) as f:
        for line in f:
            parts = line.split()
            if len(parts) < 2:
                continue
            try:
                a, b = int(parts[0]), int(parts[1])
            except ValueError:
                continue
            us.append(a - 1)
            vs.append(b - 1)
    return np.array(us, dtype=np.int64), np.array(vs, dtype=np.int64)


def write_mis_file(path, mis):
    idx = np.nonzero(np.asarray(mis))[0] + 1
    with open(path, "w") as f:
        if idx.size:
            f.write("\n".join(str(int(i)) for i in idx))
            f.write("\n")


def read_mis_file(path, n):
    out = np.zeros(n, dtype=np.uint8)
    with open(path) as f:
        for line in f:
            s = line.strip()
            if not s:
                continue
            i = int(s) - 1
            if 0 <= i < n:
                out[i] = 1
    return out
