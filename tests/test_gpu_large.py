"""The 64-bit .egr layout at more than 2^31 directed entries, through the
C-ABI.  A band graph (vertex i adjacent to every j with 0 < |i - j| <= 27)
with 41,000,000 vertices has 2,213,999,244 entries, so row offsets and entry
positions pass 2^31 and the file needs the int64-sentinel nindex.  Two batches
of 1,000,000 toggles (half deletes of band edges, half inserts of
non-adjacent pairs) run in exact-MIS mode; checked properties that hold at
any size: the rows of 2,000 sampled vertices against a host simulation of the
overlay rules, the degree sum against the counted effective updates, and an
independent, maximal membership after every batch.

About 9 GB on the device and ~30 GB of host memory: it runs only when
MISFIT_GB_LARGE=1."""
import os
import time

import numpy as np
import pytest

from misfit_gb300 import native
from misfit_gb300 import workloads as W

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(os.environ.get("MISFIT_GB_LARGE") != "1", reason="set MISFIT_GB_LARGE=1")]

N = 41_000_000
W_BAND = 27


def band_csr(n, w):
    import torch
    dev = "cuda"
    i = torch.arange(n, dtype=torch.int64, device=dev)
    d = torch.cat([torch.arange(-w, 0, device=dev), torch.arange(1, w + 1, device=dev)])
    lo = torch.clamp(i - w, min=0)
    hi = torch.clamp(i + w, max=n - 1)
    deg = (hi - lo).to(torch.int64)  # entries per row (the vertex itself excluded)
    nindex = torch.zeros(n + 1, dtype=torch.int64, device=dev)
    nindex[1:] = torch.cumsum(deg, 0)
    parts = []
    step = 1 << 22
    for a in range(0, n, step):
        ii = i[a:a + step, None] + d[None, :]
        ok = (ii >= 0) & (ii < n)
        parts.append(ii[ok].to(torch.int32).cpu())
        del ii, ok
    nlist = torch.cat(parts).numpy()
    return nindex.cpu().numpy(), nlist


def make_batch(rng, n, w, m):
    nd = m // 2
    a = rng.integers(0, n - w - 1, size=nd)
    b = a + rng.integers(1, w + 1, size=nd)
    x = rng.integers(0, n, size=m - nd)
    y = (x + rng.integers(w + 1, n - w, size=x.size)) % n
    u = np.concatenate([a, x]).astype(np.int32)
    v = np.concatenate([b, y]).astype(np.int32)
    ins = np.concatenate([np.zeros(nd, np.uint8), np.ones(m - nd, np.uint8)])
    perm = rng.permutation(m)
    return u[perm], v[perm], ins[perm]


class OverlayModel:
    """The reference's overlay rules for the band graph: adjacency, tombstones
    (a re-inserted base edge returns to its base position), added entries in
    insertion order; rows are kept only for the sampled vertices."""

    def __init__(self, n, w, sample):
        self.n, self.w = n, w
        self.dead = set()          # tombstoned base pairs (lo, hi)
        self.added = set()         # added pairs (lo, hi)
        self.sample = set(int(s) for s in sample)
        self.order = {int(s): [] for s in sample}  # added neighbours in insertion order

    def base(self, a, b):
        return a != b and abs(a - b) <= self.w

    def apply(self, u, v, ins):
        delta = 0
        for a, b, f in zip(u.tolist(), v.tolist(), ins.tolist()):
            k = (min(a, b), max(a, b))
            adj = (self.base(a, b) and k not in self.dead) or k in self.added
            if f and not adj:
                delta += 2
                if self.base(a, b):
                    self.dead.discard(k)
                else:
                    self.added.add(k)
                    for x, y in ((a, b), (b, a)):
                        if x in self.order:
                            self.order[x].append(y)
            elif not f and adj:
                delta -= 2
                if k in self.added:
                    self.added.discard(k)
                    for x, y in ((a, b), (b, a)):
                        if x in self.order:
                            self.order[x].remove(y)
                else:
                    self.dead.add(k)
        return delta

    def row(self, x):
        lo, hi = max(0, x - self.w), min(self.n - 1, x + self.w)
        base = [y for y in range(lo, hi + 1) if y != x and (min(x, y), max(x, y)) not in self.dead]
        return np.array(base + self.order[x], dtype=np.int32)


def test_int64_layout_beyond_2_31_entries(gpu_lib, tmp_path):
    t0 = time.time()
    nindex, nlist = band_csr(N, W_BAND)
    assert nlist.size > 2**31
    path = str(tmp_path / "band.egr")
    W.write_egr(path, N, nindex, nlist, wide=True)
    entries = int(nlist.size)
    del nlist
    g = native.Graph.open_egr(path)
    try:
        assert g.n == N
        mis = np.zeros(N, np.uint8)
        mis[::W_BAND + 1] = 1                   # the greedy MIS of the band graph
        g.set_mis(mis)
        assert g.check_mis() == (0, 0)
        g.set_exact(True)
        rng = np.random.default_rng(3)
        sample = rng.integers(0, N, size=2000)
        model = OverlayModel(N, W_BAND, sample)
        total = entries
        for b in range(2):
            u, v, ins = make_batch(rng, N, W_BAND, 1_000_000)
            total += model.apply(u, v, ins)
            t = time.time()
            g.apply_batch(u, v, ins)
            dt = time.time() - t
            print("batch %d: %.3f s, %.0f updates/s, sub-batches %d" % (b, dt, u.size / dt,
                                                                        g.stats()["sub_batches"]))
            assert g.check_mis() == (0, 0), b
        for x in sample.tolist():
            assert np.array_equal(g.row(x), model.row(x)), x
        assert int(g.degrees().astype(np.int64).sum()) == total
        print("total %.1f s" % (time.time() - t0))
    finally:
        g.close()
