"""CPU emulations of two lane schedules of the CUDA kernels, checked for
coverage (no GPU needed):

* the shuffle adjoint's item cursor (``AdjItems`` in
  rough-path-primitives_gb300/csrc/shuffle.cu): items (op degree m, mask M,
  u_hi, letter a), letter innermost; lane l of a warp starts at item l and
  steps 32 items at a time.  The 32 lanes together must visit every item of
  the nested (m desc, Gosper masks, u_hi, a) enumeration exactly once, and a
  single thread (start 0, step 1) must visit them in that order;
* the reverse signature pass's letter butterfly (``letter_butterfly`` /
  ``store_letter_partials`` in csrc/signature.cu): each lane holds WT
  per-letter values; after the reduce-scatter and xor levels, exactly one
  storing lane per letter must hold the warp's total of that letter.

The enumeration of masks of weight m follows Gosper's successor, as the
reference's shuffle kernels do
(include/rpp/gpu/block/operations/basic/st_adj_mul.hpp:56-100)."""
import random

import pytest


def _ffs(x):
    return (x & -x).bit_length()


def _gosper(M):
    low = M & -M
    ripple = M + low
    return ripple | (((ripple ^ M) >> 2) >> (_ffs(M) - 1))


def _cursor_items(W, nw, a0, a1, mlo, mhi, first, step):
    """The device cursor: init(first), then advance(step) until done."""
    pw = [W ** i for i in range(32)]
    out = []
    if mlo > mhi or a0 >= a1:
        return out
    st = {"a": a0, "m": mhi, "uh": 0}

    def start_degree():
        M = (1 << st["m"]) - 1
        st.update(M=M, last=M << nw, nhi=1 if st["m"] <= 1 else pw[st["m"] - 2])

    def next_mask():
        if st["M"] != st["last"]:
            st["M"] = _gosper(st["M"])
            return True
        st["m"] -= 1
        if st["m"] < mlo:
            return False
        start_degree()
        return True

    def advance(k):
        carry = k
        if a1 - a0 > 1:  # the device divides by W here (a1 - a0 = W)
            carry, r = divmod(st["a"] - a0 + k, a1 - a0)
            st["a"] = a0 + r
        st["uh"] += carry
        while st["uh"] >= st["nhi"]:
            st["uh"] -= st["nhi"]
            if not next_mask():
                return False
        return True

    start_degree()
    if not advance(first):
        return out
    while True:
        out.append((st["m"], st["M"], st["uh"], st["a"]))
        if not advance(step):
            return out


def _all_items(W, nw, a0, a1, mlo, mhi):
    pw = [W ** i for i in range(32)]
    res = []
    for m in range(mhi, mlo - 1, -1):
        nhi = 1 if m <= 1 else pw[m - 2]
        M = (1 << m) - 1
        last = M << nw
        while True:
            for uh in range(nhi):
                for a in range(a0, a1):
                    res.append((m, M, uh, a))
            if M == last:
                break
            M = _gosper(M)
    return res


@pytest.mark.parametrize("W", [1, 2, 3, 5, 8])
def test_adjoint_cursor_covers_every_item_once(W):
    for nw in range(5):
        for a0, a1 in ((0, W), (0, 1), (W - 1, W)):
            for mlo in range(3):
                for mhi in range(mlo - 1, 5):
                    want = _all_items(W, nw, a0, a1, mlo, mhi)
                    assert len(set(want)) == len(want)
                    got = []
                    for lane in range(32):
                        got += _cursor_items(W, nw, a0, a1, mlo, mhi, lane, 32)
                    assert sorted(got) == sorted(want), (W, nw, a0, a1, mlo, mhi)
                    assert _cursor_items(W, nw, a0, a1, mlo, mhi, 0, 1) == want


def _butterfly(vals, WT):
    """letter_butterfly + store_letter_partials over one warp; returns
    {letter: stored value}."""
    v = [list(x) for x in vals]
    base, cnt = [0] * 32, [WT] * 32
    K, off = WT, 16
    while K > 1:
        h = (K + 1) // 2
        send = []
        for lane in range(32):
            up = bool(lane & off)
            send.append([v[lane][i] if up else (v[lane][h + i] if h + i < K else 0.0) for i in range(h)])
        nv = []
        for lane in range(32):
            up = bool(lane & off)
            keep = [(v[lane][h + i] if h + i < K else 0.0) if up else v[lane][i] for i in range(h)]
            nv.append([keep[i] + send[lane ^ off][i] for i in range(h)])
            if up:
                base[lane] += h
                cnt[lane] = max(cnt[lane] - h, 0)
            else:
                cnt[lane] = min(cnt[lane], h)
        v, K, off = nv, h, off >> 1
    x = [row[0] for row in v]
    while off > 0:
        x = [x[lane] + x[lane ^ off] for lane in range(32)]
        off >>= 1
    halvings = 0 if WT <= 1 else 1 if WT <= 2 else 2 if WT <= 4 else 3 if WT <= 8 else 4
    stored = {}
    for lane in range(32):
        if cnt[lane] > 0 and (lane & ((32 >> halvings) - 1)) == 0:
            assert base[lane] not in stored, "two lanes store one letter"
            stored[base[lane]] = x[lane]
    return stored


@pytest.mark.parametrize("WT", range(1, 9))
def test_letter_butterfly_stores_each_letter_total_once(WT):
    rng = random.Random(WT)
    vals = [[rng.uniform(-1, 1) for _ in range(WT)] for _ in range(32)]
    stored = _butterfly(vals, WT)
    assert sorted(stored) == list(range(WT))
    for a in range(WT):
        assert stored[a] == pytest.approx(sum(vals[lane][a] for lane in range(32)), rel=1e-12, abs=1e-12)
