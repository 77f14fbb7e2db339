"""GPU: the Fitch pair entry points touch exactly the bytes of the sites.

The reference's vectors hold exactly `chars` elements (bv_malloc,
lib/bitvector/bv.c:32-42), so a BV8 stub hands pgpu_fitch_median2 a buffer of
n_sites bytes and a BV16 stub one of 2 n_sites bytes, neither padded to whole
32-bit words.  Each buffer here is an exact-size bytearray followed by canary
bytes; all three pair entry points must leave the canaries alone and give the
oracle's medians and counts (the oracle's two-tip Fitch postorder is the pair
median with its union count).
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CANARY = bytes([0xA5, 0x5A, 0xC3, 0x3C] * 4)


def _buf(payload: bytes):
    raw = bytearray(payload + CANARY)
    return raw, (C.c_char * len(raw)).from_buffer(raw)


def _masks(rng, n, lb):
    hi = (1 << lb) - 1
    # small sets so that some intersections are empty
    bits = rng.integers(0, lb, (n, 2))
    return ((np.uint64(1) << bits[:, 0].astype(np.uint64)) |
            (np.uint64(1) << bits[:, 1].astype(np.uint64))).astype(np.uint64) & np.uint64(hi)


@pytest.mark.parametrize("lb", [8, 16])
@pytest.mark.parametrize("n_sites", list(range(1, 10)))
def test_pair_calls_stay_inside_exact_size_buffers(ctx, orc, lb, n_sites):
    dt = np.uint8 if lb == 8 else np.uint16
    rng = np.random.default_rng(100 * lb + n_sites)
    a = _masks(rng, n_sites, lb).astype(dt)
    b = _masks(rng, n_sites, lb).astype(dt)
    w = rng.integers(1, 9, n_sites, dtype=np.uint32)
    # oracle: the two-tip postorder over the same packed words
    pack = lambda x: np.frombuffer(x.tobytes() + bytes(-len(x.tobytes()) % 4), np.uint32)
    tips = np.stack([pack(a), pack(b)])
    med, sc, tot_w, _ = orc.fitch_tree_packed([0], [1], tips, n_sites, lb, w)
    _, _, count, _ = orc.fitch_tree_packed([0], [1], tips, n_sites, lb, None)
    exp_bytes = med[0].tobytes()[: a.nbytes]

    ra, pa = _buf(a.tobytes())
    rb, pb = _buf(b.tobytes())
    rw, pw = _buf(w.tobytes())
    for mode in ("median2", "weighted", "distance"):
        ro, po = _buf(bytes([0xEE]) * a.nbytes)
        res = C.c_uint64(12345)
        if mode == "median2":
            ctx.call("pgpu_fitch_median2", C.addressof(pa), C.addressof(pb), C.addressof(po),
                     n_sites, lb, C.byref(res))
            assert res.value == count
        elif mode == "weighted":
            ctx.call("pgpu_fitch_median2_weighted", C.addressof(pa), C.addressof(pb),
                     C.addressof(pw), C.addressof(po), n_sites, lb, C.byref(res))
            assert res.value == tot_w
        else:
            ctx.call("pgpu_fitch_distance", C.addressof(pa), C.addressof(pb), n_sites, lb,
                     C.byref(res))
            assert res.value == count
        if mode != "distance":
            assert bytes(ro[: a.nbytes]) == exp_bytes, f"{mode}: median differs from the oracle"
        else:
            assert bytes(ro[: a.nbytes]) == bytes([0xEE]) * a.nbytes, "distance wrote its output"
        assert bytes(ro[a.nbytes:]) == CANARY, f"{mode}: wrote past the output buffer"
        for r, n in ((ra, a.nbytes), (rb, b.nbytes), (rw, w.nbytes)):
            assert bytes(r[n:]) == CANARY, f"{mode}: an input's canary changed"
    # the inputs are unchanged too
    assert bytes(ra[: a.nbytes]) == a.tobytes() and bytes(rb[: b.nbytes]) == b.tobytes()


def test_pair_matches_reference_build_where_present(ctx):
    """Where the reference's own bv.c was built (oracle/_ref), the exact-size
    BV8 call also matches its bv_fitch bit for bit."""
    import oracle
    ref = oracle.ref_lib(8)
    if ref is None:
        pytest.skip("the reference's bv.c is built only where its tree exists")
    rng = np.random.default_rng(7)
    for n in range(1, 10):
        a = _masks(rng, n, 8).astype(np.uint8)
        b = _masks(rng, n, 8).astype(np.uint8)
        out_ref = np.zeros(n, np.uint8)
        cnt_ref = ref.bvref_fitch_median2(a.ctypes.data, b.ctypes.data, out_ref.ctypes.data, n)
        ra, pa = _buf(a.tobytes())
        rb, pb = _buf(b.tobytes())
        ro, po = _buf(bytes(n))
        res = C.c_uint64(0)
        ctx.call("pgpu_fitch_median2", C.addressof(pa), C.addressof(pb), C.addressof(po), n, 8,
                 C.byref(res))
        assert res.value == cnt_ref and bytes(ro[:n]) == out_ref.tobytes()
        assert bytes(ro[n:]) == CANARY
