"""Oracle: CPU restatements of phylocaml's hot path -- TEST INFRASTRUCTURE.

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline and
reference legs may use this package, and only as the checker or the timed CPU
baseline, never as the product path.

  liboracle.so   (fitch_oracle.c, prune_oracle.c)   my C restatements
  _ref/libbvref_wN.so                               phylocaml's own bv.c,
                                                    compiled where the
                                                    reference tree exists
  mlmodel_oracle.py                                 MlModel / mlmodel.c in numpy+LAPACK

Parity of the Fitch restatement is pinned against the reference's compiled
bv.c and the DNA code-pair table of test/costMatrixTest.ml:83-108; the
P-matrix restatement against scipy's LAPACK (the routines mlmodel.c calls)
and analytic identities; the pruning restatement against brute-force
enumeration of ancestral states.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIBORACLE = HERE / "_build" / "liboracle.so"
REF_DIR = HERE / "_ref"
# the phylocaml checkout: $PHYLOCAML_REF, else a directory named `reference`
# beside this repository
REFERENCE_TREE = Path(os.environ.get("PHYLOCAML_REF", str(HERE.parent.parent / "reference")))

_I32P = C.POINTER(C.c_int32)
_P = C.c_void_p
_U64 = C.c_uint64


def build(quiet: bool = True) -> None:
    """Compiles liboracle.so, and the reference's bv.c when its tree exists."""
    cmd = ["make", "-C", str(HERE), "oracle"]
    if (REFERENCE_TREE / "lib" / "bitvector" / "bv.c").exists():
        cmd = ["make", "-C", str(HERE), "all", f"REF={REFERENCE_TREE}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stdout}\n{r.stderr}")
    if not quiet:
        print(r.stdout)


_orc = None


def lib() -> C.CDLL:
    global _orc
    if _orc is None:
        if not LIBORACLE.exists():
            build()
        L = C.CDLL(str(LIBORACLE))
        L.orc_bv8_fitch.restype = _U64
        L.orc_bv8_fitch.argtypes = [_P, _P, _P, _U64]
        L.orc_bv8_distance.restype = _U64
        L.orc_bv8_distance.argtypes = [_P, _P, _U64]
        L.orc_bv8_fitch_tree_alloc.restype = _U64
        L.orc_bv8_fitch_tree_alloc.argtypes = [C.c_int32, _P, _P, _P, _U64, _P]
        L.orc_bv8_fitch_tree_alloc_mt.restype = _U64
        L.orc_bv8_fitch_tree_alloc_mt.argtypes = [C.c_int32, _P, _P, _P, _U64, _P, C.c_int]
        L.orc_nonadditive_median2.restype = C.c_double
        L.orc_nonadditive_median2.argtypes = [_P, _P, _P, _U64, _P]
        L.orc_fitch_tree_packed.restype = C.c_int
        L.orc_fitch_tree_packed.argtypes = [C.c_int32, _P, _P, _P, _U64, _U64, C.c_int, _P, _P,
                                            _P, _P, _P]
        L.orc_prune_lnl.restype = C.c_int
        L.orc_prune_lnl.argtypes = [C.c_int32, _P, _P, _P, C.c_int, C.c_int, _P, _P, _P, C.c_int,
                                    _P, _P, _U64, _P, _P, C.c_int]
        _orc = L
    return _orc


def _p(a):
    return None if a is None else a.ctypes.data


def ref_lib(width: int):
    """phylocaml's own bv.c for element width 8/16/32/64, or None if it was
    not built (the reference tree is absent on this machine)."""
    path = REF_DIR / f"libbvref_w{width}.so"
    if not path.exists():
        return None
    L = C.CDLL(str(path))
    for name, res, args in [
        ("bvref_width", C.c_int, []),
        ("bvref_fitch_median2", _U64, [_P, _P, _P, _U64]),
        ("bvref_distance", _U64, [_P, _P, _U64]),
        ("bvref_union", None, [_P, _P, _P, _U64]),
        ("bvref_inter", None, [_P, _P, _P, _U64]),
        ("bvref_fitch_tree", C.c_int, [C.c_int32, _P, _P, _P, _U64, _P, _P]),
        ("bvref_fitch_tree_alloc", _U64, [C.c_int32, _P, _P, _P, _U64, _P]),
        ("bvref_fitch_tree_alloc_mt", _U64, [C.c_int32, _P, _P, _P, _U64, _P, C.c_int]),
    ]:
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    assert L.bvref_width() == width
    return L


# ---- Python-side helpers over the C restatements ---------------------------

def fitch_tree_packed(left, right, tip_words, n_sites, lane_bits, weights=None):
    """orc_fitch_tree_packed: (node_sets, site_cost, total, node_counts)."""
    left = np.ascontiguousarray(left, np.int32)
    right = np.ascontiguousarray(right, np.int32)
    tip_words = np.ascontiguousarray(tip_words, np.uint32)
    n_tips = len(left) + 1
    ld = tip_words.shape[1]
    node_sets = np.zeros((n_tips - 1, ld), np.uint32)
    site_cost = np.zeros(n_sites, np.uint32)
    node_counts = np.zeros(n_tips - 1, np.uint64)
    total = C.c_uint64(0)
    w = None if weights is None else np.ascontiguousarray(weights, np.uint32)
    rc = lib().orc_fitch_tree_packed(n_tips, _p(left), _p(right), _p(tip_words), ld, n_sites,
                                     lane_bits, _p(w), _p(node_sets), _p(site_cost),
                                     C.byref(total), _p(node_counts))
    if rc != 0:
        raise ValueError("orc_fitch_tree_packed: bad arguments")
    return node_sets, site_cost, int(total.value), node_counts


def bv8_fitch_tree(left, right, tip_bytes, n_threads=1):
    """The restated bv_fitch postorder (one char per byte, allocating path):
    (internal state bytes [n_int, chars], summed union count)."""
    left = np.ascontiguousarray(left, np.int32)
    right = np.ascontiguousarray(right, np.int32)
    tip_bytes = np.ascontiguousarray(tip_bytes, np.uint8)
    n_tips, chars = tip_bytes.shape
    out = np.zeros((n_tips - 1, chars), np.uint8)
    if n_threads > 1:
        tot = lib().orc_bv8_fitch_tree_alloc_mt(n_tips, _p(left), _p(right), _p(tip_bytes), chars,
                                                _p(out), n_threads)
    else:
        tot = lib().orc_bv8_fitch_tree_alloc(n_tips, _p(left), _p(right), _p(tip_bytes), chars,
                                             _p(out))
    return out, int(tot)


def nonadditive_median2(xs, ys, weights):
    xs = np.ascontiguousarray(xs, np.int64)
    ys = np.ascontiguousarray(ys, np.int64)
    w = np.ascontiguousarray(weights, np.float64)
    out = np.empty_like(xs)
    cost = lib().orc_nonadditive_median2(_p(xs), _p(ys), _p(w), len(xs), _p(out))
    return out, float(cost)


def prune_lnl(left, right, P, pi, probs, tip_codes, code_table, weights, n_threads=1,
              site_lnl=False):
    """orc_prune_lnl: FP64 lnL (and per-site lnL when asked).
    P: [2n-2, R, S, S] float64; tip_codes: [n_tips, n_pat] uint8;
    code_table: [n_codes, S] float64."""
    left = np.ascontiguousarray(left, np.int32)
    right = np.ascontiguousarray(right, np.int32)
    P = np.ascontiguousarray(P, np.float64)
    pi = np.ascontiguousarray(pi, np.float64)
    probs = np.ascontiguousarray(probs, np.float64)
    tip_codes = np.ascontiguousarray(tip_codes, np.uint8)
    code_table = np.ascontiguousarray(code_table, np.float64)
    w = None if weights is None else np.ascontiguousarray(weights, np.float64)
    n_tips, n_pat = tip_codes.shape
    R, S = P.shape[1], P.shape[2]
    sl = np.empty(n_pat, np.float64) if site_lnl else None
    out = C.c_double(0.0)
    rc = lib().orc_prune_lnl(n_tips, _p(left), _p(right), _p(P), S, R, _p(pi), _p(probs),
                             _p(tip_codes), code_table.shape[0], _p(code_table), _p(w), n_pat,
                             _p(sl), C.byref(out), n_threads)
    if rc != 0:
        raise ValueError(f"orc_prune_lnl failed ({rc})")
    return (out.value, sl) if site_lnl else out.value
