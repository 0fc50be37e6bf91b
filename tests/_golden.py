"""Loading helpers for the committed golden fixtures."""
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
NAMES = ["sample", "er1500", "rmat10", "rmat10g"]


def load(name):
    d = np.load(os.path.join(GOLDEN, name + ".npz"))
    return {k: d[k] for k in d.files}


def batches(g):
    return [(g["b%d_u" % i], g["b%d_v" % i], g["b%d_ins" % i]) for i in range(int(g["num_batches"]))]


def rows(g, i):
    ptr, idx = g["b%d_rows_ptr" % i], g["b%d_rows_idx" % i]
    return [idx[ptr[x]:ptr[x + 1]] for x in range(int(g["n"]))]


def twohop(g, i):
    seeds = g["b%d_2hop_seeds" % i]
    ptr, idx = g["b%d_2hop_ptr" % i], g["b%d_2hop_idx" % i]
    return [(int(s), idx[ptr[k]:ptr[k + 1]]) for k, s in enumerate(seeds)]


# Fixtures carrying the reference engine's own results (its sync engine and
# both main() binaries run on the CPU): the four streams above and config 1.
REF_NAMES = NAMES + ["cfg1"]


def n_of(g):
    return int(g["n"])


def mis0(g):
    m = g["mis0"]
    return np.unpackbits(m)[: n_of(g)] if m.size != n_of(g) else m


def mis_ref(g, i, serial=False):
    """Membership after batch i from the reference's sync engine (bulk-
    synchronous clustering unless serial)."""
    return np.unpackbits(g["b%d_mis_ref%s" % (i, "_serial" if serial else "")])[: n_of(g)]


def main_final_mis(g, engine):
    """Final-MIS file of the reference's bin/misfit (engine "sync") or
    bin/misfit_async ("async") main() over the whole stream."""
    return np.unpackbits(g["main_%s_final_mis" % engine])[: n_of(g)]


def cid_sha(cids):
    import hashlib
    return hashlib.sha256(np.ascontiguousarray(cids, dtype="<i4").tobytes()).digest()


def initial_max_csr(g):
    return int(g["max_csr"]) if "max_csr" in g else int(g["initial_max_csr"])
