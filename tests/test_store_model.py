"""CPU model of the 16-byte tile store of the keys-only merge kernel
(store_tile / vec_shift in gpu-mms_gb300/csrc/gms_kernels.cuh).

The last merge level writes a tile of cnt keys into a 16-byte-aligned shared
buffer starting vs keys in, vs being the tile's destination offset within its
16-byte line of global memory (in keys).  store_tile then copies keys
[0, h) and [tail0, cnt) one by one and [h, tail0) as 16-byte vectors.  The
model replays that index arithmetic for every line offset, key size and tile
length a tile can have and checks that:
  * every key of [0, cnt) is written exactly once, and nothing outside it;
  * every vector access is 16-byte aligned on both sides (shared at byte
    (vs + q) * size of the buffer, global at the destination address);
  * the threads' loops (t0, t0 + nthr, ...) cover the scalar and vector work.
"""
import pytest


def store_plan(g_addr, size, cnt):
    """Accesses of store_tile for a destination byte address g_addr."""
    e = 16 // size
    mis = (g_addr // size) % e  # vec_shift
    h = min(cnt, (e - mis) % e)
    nvec = (cnt - h) // e
    tail0 = h + nvec * e
    nscal = h + (cnt - tail0)
    scalars = [j if j < h else tail0 + (j - h) for j in range(nscal)]
    vectors = [h + e * v for v in range(nvec)]
    return mis, scalars, vectors, e


@pytest.mark.parametrize("size", [4, 8])
def test_store_tile_covers_each_key_once_aligned(size):
    e = 16 // size
    for line_off in range(e):  # destination offset within its 16-byte line
        g_base = 4096 + line_off * size
        for cnt in list(range(0, 70)) + [8431, 8432, 4079, 4080]:
            vs, scalars, vectors, e_ = store_plan(g_base, size, cnt)
            assert vs == line_off
            written = list(scalars)
            for q in vectors:
                # shared: buffer 16-byte aligned, the tile starts vs keys in
                assert ((vs + q) * size) % 16 == 0, (size, line_off, cnt, q)
                assert (g_base + q * size) % 16 == 0, (size, line_off, cnt, q)
                written.extend(range(q, q + e_))
            assert sorted(written) == list(range(cnt)), (size, line_off, cnt)
            # at most E-1 single keys at each end
            assert len(scalars) <= 2 * (e_ - 1)


def test_store_tile_thread_loops_cover_work():
    size, cnt = 4, 8432
    for line_off in range(4):
        _, scalars, vectors, _ = store_plan(4096 + 4 * line_off, size, cnt)
        for nthr, t_first in [(288, 0), (256, 32)]:  # all threads; all but warp 0 (persistent CTA)
            seen_s, seen_v = [], []
            for t in range(t_first, t_first + nthr):
                t0 = t - t_first
                seen_s += list(range(t0, len(scalars), nthr))
                seen_v += list(range(t0, len(vectors), nthr))
            assert sorted(seen_s) == list(range(len(scalars)))
            assert sorted(seen_v) == list(range(len(vectors)))


def test_shifted_tile_fits_merge_buffer():
    # the last level's output [vs, vs + cnt) plus the spill of its last window
    # (ITEMS - 1 keys) must fit the merge buffer of MergeSmemLayout:
    # TMAX + (kMaxK/2) * GAP + ITEMS + 4 keys (288 x 31 and 256 x 17 geometries)
    for nt, items, gap, size in [(288, 31, 32, 4), (256, 17, 18, 8)]:
        tmax = (nt - 16) * items
        cap_keys = tmax + 16 * gap + items + 4
        e = 16 // size
        assert (e - 1) + tmax + (items - 1) <= cap_keys
