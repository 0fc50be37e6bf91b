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
