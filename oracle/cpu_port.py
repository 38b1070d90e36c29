"""ctypes driver of the C restatement (oracle/pmm_oracle.c) -- TEST
INFRASTRUCTURE: the CPU baseline leg of bench.py and a cross-check of the
NumPy oracle in tests.  Builds oracle/_lib/libpmm_oracle.so with gcc/OpenMP."""
import ctypes as C
import os
import subprocess
import time

import numpy as np

from . import pmm_oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_lib", "libpmm_oracle.so")
_lib = None


def build():
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    cmd = ["gcc", "-O2", "-fopenmp", "-shared", "-fPIC", "-std=gnu11",
           os.path.join(HERE, "pmm_oracle.c"), "-o", LIB + ".tmp", "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle C build failed:\n" + r.stderr)
    os.replace(LIB + ".tmp", LIB)
    return LIB


class OraTree(C.Structure):
    _fields_ = [("N", C.c_int), ("n", C.c_int), ("K", C.c_int), ("c0", C.c_void_p),
                ("c1", C.c_void_p), ("parent", C.c_void_p), ("chars", C.c_void_p),
                ("kc", C.c_void_p), ("q", C.c_void_p), ("kmax", C.c_int), ("d", C.c_void_p),
                ("nu", C.c_double), ("phi", C.c_double), ("llh", C.c_double)]


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        L = C.CDLL(LIB)
        L.ora_em.restype = C.c_double
        L.ora_em.argtypes = [C.POINTER(OraTree), C.c_int, C.c_int, C.c_int]
        L.ora_loglik.restype = None
        L.ora_loglik.argtypes = [C.POINTER(OraTree), C.c_int]
        L.ora_site_loglik.restype = None
        L.ora_site_loglik.argtypes = [C.POINTER(OraTree), C.c_void_p]
        L.ora_num_threads.restype = C.c_int
        _lib = L
    return _lib


def _prepare(newicks, rows, Q, leaf_order, nu, phi, ds=None, enc=None):
    keep = []
    trees = (OraTree * len(newicks))()
    if enc is None:
        enc = O.recode([rows[c] for c in leaf_order], Q, compat=True)
    chars = np.ascontiguousarray(enc.chars, np.int32)
    kc = np.ascontiguousarray(enc.k, np.int32)
    q = np.ascontiguousarray(enc.q, np.float64)
    keep += [chars, kc, q]
    for i, nw in enumerate(newicks):
        tr = O.parse_tree(nw, leaf_order)
        c0 = np.array([c[0] if c else -1 for c in tr.children], np.int32)
        c1 = np.array([c[1] if c else -1 for c in tr.children], np.int32)
        par = tr.parent.astype(np.int32)
        d = (tr.branch_lengths if ds is None else ds[i]).astype(np.float64).copy()
        keep += [c0, c1, par, d]
        trees[i] = OraTree(len(par), tr.num_leaves, chars.shape[1], c0.ctypes.data,
                           c1.ctypes.data, par.ctypes.data, chars.ctypes.data, kc.ctypes.data,
                           q.ctypes.data, q.shape[1], d.ctypes.data, nu, phi, 0.0)
    return trees, keep


def em(newicks, rows, Q, leaf_order, nu=0.5, phi=0.5, iters=1, rounds=4):
    """Run `iters` EM iterations per tree; returns (llh, nu, phi, d list, seconds)."""
    trees, keep = _prepare(newicks, rows, Q, leaf_order, nu, phi)
    t = lib().ora_em(trees, len(newicks), iters, rounds)
    ds = [np.ctypeslib.as_array(C.cast(trees[i].d, C.POINTER(C.c_double)),
                                shape=(trees[i].N,)).copy() for i in range(len(newicks))]
    return ([trees[i].llh for i in range(len(newicks))], [trees[i].nu for i in range(len(newicks))],
            [trees[i].phi for i in range(len(newicks))], ds, t)


def loglik(newicks, rows, Q, leaf_order, nu, phi, ds=None):
    """fastEM log-likelihood of every tree at (d, nu, phi), one tree per core;
    ``ds``: branch lengths per tree in the parse_tree numbering (default: the
    newick's)."""
    trees, keep = _prepare(newicks, rows, Q, leaf_order, nu, phi, ds)
    lib().ora_loglik(trees, len(newicks))
    return np.array([trees[i].llh for i in range(len(newicks))])


def site_loglik(newick, rows, Q, leaf_order, nu, phi, d=None, enc=None):
    """Per-site fastEM log-likelihood of one tree (original site order), sites
    in parallel: the form that fits 50,000-leaf x 300-site trees."""
    if enc is None:
        enc = O.recode([rows[c] for c in leaf_order], Q, compat=True)
    trees, keep = _prepare([newick], rows, Q, leaf_order, nu, phi,
                           None if d is None else [np.asarray(d)], enc)
    out = np.zeros(enc.chars.shape[1])
    lib().ora_site_loglik(trees, out.ctypes.data)
    return out


def em_throughput(workload, n_trees, iters):
    """Tree-EM-iterations per second of the C restatement on the first
    ``n_trees`` candidates of a workload, all host cores."""
    nw = workload.newicks[:n_trees]
    _, _, _, _, t = em(nw, workload.rows, workload.Q, workload.leaf_order, 0.5, 0.5, iters)
    return n_trees * iters / t, int(lib().ora_num_threads())
