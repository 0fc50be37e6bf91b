"""Batch files parsed on the device (mf_parse_batch_file) against the host
parser (mf_read_batch_file) plus mf_flag_updates: same lines kept, same ids,
same flags, bit for bit."""
import numpy as np
import pytest

from misfit_gb300 import native
from misfit_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _host(g, path):
    u, v = native.read_batch_file(path, g.n)
    return u, v, g.flag_updates(u, v)


TRICKY = (
    "%%MatrixMarket matrix coordinate pattern general\n"
    "% a comment\n"
    "\n"
    "1 2\n"
    "3\t4\r\n"
    "  5   6   extra 7\n"
    "+7 8\n"
    "-1 2\n"
    "9 9\n"
    "0 3\n"
    "10 100000000\n"
    "2147483648 3\n"
    "11 99999999999999999999\n"
    "12x 13\n"
    "14 15y\n"
    "16,17\n"
    "18 -\n"
    "19\n"
    "20 21 22\n"
    "0021 0022\n"
    "\t\r\n"
    "23 24"
)


def test_parse_rules_match_host(gpu_lib, tmp_path):
    nindex, nlist = W.er_graph(500, 6, 3)
    g = native.Graph.from_csr(nindex, nlist)
    try:
        path = str(tmp_path / "1.mtx")
        with open(path, "w", newline="") as f:
            f.write(TRICKY)
        hu, hv, hi = _host(g, path)
        du, dv, di = g.parse_batch_file(path)
        assert hu.size > 5
        assert np.array_equal(du, hu) and np.array_equal(dv, hv) and np.array_equal(di, hi)
        empty = str(tmp_path / "2.mtx")
        open(empty, "w").close()
        du, dv, di = g.parse_batch_file(empty)
        assert du.size == 0
        with pytest.raises(native.MisfitError):
            g.parse_batch_file(str(tmp_path / "missing.mtx"))
    finally:
        g.close()


def test_parse_large_random_file(gpu_lib, tmp_path):
    n = 50000
    nindex, nlist = W.er_graph(n, 10, 5)
    g = native.Graph.from_csr(nindex, nlist)
    try:
        ts = W.ToggleStream(n, nindex, nlist, 6)
        u, v = ts.next_batch(300000)
        path = str(tmp_path / "3.mtx")
        W.write_batch_file(path, u, v)
        hu, hv, hi = _host(g, path)
        du, dv, di = g.parse_batch_file(path)
        assert hu.size == u.size
        assert np.array_equal(du, hu) and np.array_equal(dv, hv) and np.array_equal(di, hi)
    finally:
        g.close()
