"""CPU model of the sentinel-padded merge windows (merge_window CHECK 2 in
gpu-mms_gb300/csrc/gms_device.cuh).

Keys-only merges under the default order pad both runs of a pair with
sentinels (the largest key) and step without run-end checks.  The model
replays a window exactly as the kernel does -- exact co-rank of each stream
by merge path, then H unchecked steps per stream that take A on ties and load
the key after the one taken -- and checks, on inputs full of largest keys and
ties, for both cursors of the kernel (MergeCursor::step_inner, which keeps A
and B apart and takes A on ties, and MergeCursorSw, which keeps the two heads
unordered and takes its first slot on ties):
  * the emitted values of every window equal the exact merge's at the same
    output positions (bit-exact output);
  * outputs past the pair's end (the spill into the gap) are all sentinels;
  * no step reads more than RunPad::read slots past a run's end, and the
    spill stays within RunPad::gap.
"""
import numpy as np
import pytest

MAXK = 0xFFFFFFFF


def run_pad(items, ns):
    read = (items + ns - 1) // ns + 1
    return read, max(read, items - 1)


def merge_path(a, b, diag, lo, hi):
    # number of A keys among the first `diag` outputs (A wins ties)
    while lo < hi:
        mid = (lo + hi) // 2
        if a[mid] <= b[diag - 1 - mid]:
            lo = mid + 1
        else:
            hi = mid
    return lo


def window(a, b, diag, items, ns, read, swap):
    na, nb = len(a), len(b)
    ap = np.concatenate([a, np.full(read, MAXK, dtype=np.uint64)])
    bp = np.concatenate([b, np.full(read, MAXK, dtype=np.uint64)])
    h = (items + ns - 1) // ns
    iq = [merge_path(a, b, diag, max(0, diag - nb), min(diag, na))]
    dq = [diag]
    for q in range(1, ns):
        d = min(diag + q * h, na + nb)
        lo = max(d - nb, iq[-1])
        hi = min(iq[-1] + h, na, d)
        iq.append(merge_path(a, b, d, lo, hi))
        dq.append(d)
    out = [None] * items
    max_over = 0
    for q in range(ns):
        if swap:
            # MergeCursorSw: slots (run, position) in either order
            c1, c2 = [ap, iq[q], na], [bp, dq[q] - iq[q], nb]
            for i in range(h):
                pos = q * h + i
                if pos >= items:
                    break
                k1, k2 = c1[0][c1[1]], c2[0][c2[1]]
                if k2 < k1:
                    c1, c2 = c2, c1
                out[pos] = c1[0][c1[1]]
                c1[1] += 1  # advance the taken cursor and load its next key
                _ = c1[0][c1[1]]
                max_over = max(max_over, c1[1] - c1[2] + 1)
            continue
        xa, xb = iq[q], dq[q] - iq[q]
        ka, kb = ap[xa], bp[xb]
        for i in range(h):
            pos = q * h + i
            if pos >= items:
                break
            ta = not (kb < ka)
            o = ka if ta else kb
            if ta:
                xa += 1
                ka = ap[xa]  # the key after the one taken
                max_over = max(max_over, xa - na + 1)
            else:
                xb += 1
                kb = bp[xb]
                max_over = max(max_over, xb - nb + 1)
            out[pos] = o
    return out, max_over


@pytest.mark.parametrize("swap", [False, True])
@pytest.mark.parametrize("items,ns", [(31, 1), (31, 2), (33, 2), (65, 1), (65, 2), (17, 1), (17, 2)])
def test_sentinel_windows_match_exact_merge(items, ns, swap):
    rng = np.random.default_rng(items * 10 + ns)
    read, gap = run_pad(items, ns)
    for trial in range(60):
        na, nb = rng.integers(0, 200, 2)
        kind = trial % 4
        if kind == 0:
            vals = rng.integers(0, 1 << 32, na + nb, dtype=np.uint64)
        elif kind == 1:  # many largest keys (equal to the sentinel)
            vals = np.where(rng.random(na + nb) < 0.5, MAXK, rng.integers(0, 8, na + nb)).astype(np.uint64)
        elif kind == 2:  # all largest keys
            vals = np.full(na + nb, MAXK, dtype=np.uint64)
        else:  # few distinct values
            vals = rng.integers(0, 3, na + nb).astype(np.uint64) * (MAXK // 2)
        a = np.sort(vals[:na])
        b = np.sort(vals[na:])
        exact = np.sort(np.concatenate([a, b]), kind="stable")
        n = na + nb
        for diag in range(0, n, items):
            m = min(items, n - diag)
            out, over = window(a, b, diag, items, ns, read, swap)
            assert over <= read, (items, ns, over, read)
            assert [int(x) for x in out[:m]] == [int(x) for x in exact[diag:diag + m]]
            assert all(int(x) == MAXK for x in out[m:])  # spill: sentinels only
            assert items - m <= gap


def test_pad_sizes():
    # the kernel instantiations: data rounds 288 x 31 and 256 x 17 (64-bit
    # keys), one stream; base-case levels 65 keys per window (32-bit keys)
    # and 33 (64-bit keys), two streams
    assert run_pad(31, 1) == (32, 32)
    assert run_pad(17, 1) == (18, 18)
    assert run_pad(65, 2) == (34, 64)
    assert run_pad(33, 2) == (18, 32)
