"""CPU model of the round/tile index arithmetic of the CUDA library.

Not the oracle: this restates the library's OWN plan (gpu-mms_gb300/csrc/
gms_sort.cuh: Engine::round / Engine::sort) and the index math of
splitter_kernel and tile_kernel (gms_kernels.cuh) in numpy, so that the
bounds every launch relies on -- above all "a tile never holds more than CAP
keys", which sizes the shared-memory buffer -- can be checked on the CPU for
any geometry (CAP, K, B) and any input distribution before code runs on a GPU.
"""
import numpy as np


def ceil_div(a, b):
    return -(-a // b)


class Geometry:
    """cap: one-CTA group capacity (GROUP mode when K*L <= cap); base:
    base-case tile (defaults to cap).  With nt/items (the merge kernel's
    threads and keys per thread) forecast tiles are cut for the window-aligned
    capacity (nt - 16) * items (WindowCap in gms_kernels.cuh), and every tile
    is checked to need at most nt windows at every merge level; without them
    tiles are cut for cap."""

    def __init__(self, cap, k, b, base=None, nt=None, items=None, sample=None):
        self.cap, self.k, self.b = cap, k, b
        self.base = base or cap
        self.nt, self.items = nt, items
        self.tile_cap = (nt - 16) * items if nt else cap
        self.g = self.tile_cap // b - k
        assert self.g > 0, "tile geometry needs TILE_CAP/B > K"
        # geometry of the rounds that merge a block sample with its positions
        # (Engine's index geometry); defaults to this one
        self.sample = sample or self


def windows_per_level(seg_lens, items):
    """Threads the window-aligned merge levels of one tile use: at the level
    with `span` segments per pair, sum over pairs of ceil(len / items)."""
    k = len(seg_lens)
    out = []
    span = 2
    while True:
        tot = 0
        for p in range(0, k, span):
            tot += ceil_div(int(sum(seg_lens[p:p + span])), items)
        out.append(tot)
        if span >= k:
            break
        span *= 2
    return out


def _stable_merge(keys, idx):
    order = np.argsort(keys, kind="stable")
    return keys[order], idx[order]


def model_round(keys, idx, L, geo, stats, level=0):
    """One K-way round over runs of length L.  Returns merged (keys, idx).

    Mirrors Engine::round: GROUP mode when K*L <= CAP, else sample -> recursive
    merge of the sample with its positions -> boundaries -> tiles.
    """
    n = len(keys)
    k, B, cap, G = geo.k, geo.b, geo.cap, geo.g
    out_k = np.empty_like(keys)
    out_i = np.empty_like(idx)
    if k * L <= cap:
        for gb in range(0, n, k * L):
            ge = min(n, gb + k * L)
            assert ge - gb <= cap
            out_k[gb:ge], out_i[gb:ge] = _stable_merge(keys[gb:ge], idx[gb:ge])
        stats["group_launches"] = stats.get("group_launches", 0) + 1
        return out_k, out_i
    runs = ceil_div(n, L)
    Ls = ceil_div(L, B)
    ns = (runs - 1) * Ls + ceil_div(n - (runs - 1) * L, B)
    # block sample: run r, block b -> slot r*Ls + b (gather_sample_kernel)
    S = np.empty(ns, dtype=keys.dtype)
    for r in range(runs):
        rs, re = r * L, min(n, (r + 1) * L)
        samp = keys[rs:re:B]
        S[r * Ls:r * Ls + len(samp)] = samp
        if r < runs - 1:
            assert len(samp) == Ls
    fk, fi = model_round(S, np.arange(ns, dtype=np.int64), Ls, geo.sample, stats, level + 1)
    groups = ceil_div(n, L * k)
    tiles_full = ceil_div(k * Ls, G)
    last_ns = ns - (groups - 1) * k * Ls
    tiles_last = ceil_div(last_ns, G)
    max_tile = 0
    for g in range(groups):
        gbase = g * L * k
        ng = min(L * k, n - gbase)
        jg = tiles_last if g == groups - 1 else tiles_full
        desc = np.zeros((jg + 1, k), dtype=np.int64)
        lens = [max(0, min((kk + 1) * L, ng) - min(kk * L, ng)) for kk in range(k)]
        # interior boundaries j = 1 .. jg-1: the first key of block F[j*G]
        js = np.arange(1, jg, dtype=np.int64)
        fpos = g * k * Ls + js * G
        assert len(js) == 0 or fpos[-1] < len(fk)
        v = fk[fpos]
        sidx = fi[fpos].astype(np.int64)
        rr = sidx // Ls
        kb = rr - g * k
        ib = (sidx - rr * Ls) * B
        assert np.all((kb >= 0) & (kb < k))
        # splitter_kernel's backward scan of F's index stream: run kk's block
        # count before boundary j is one more than the block index of run
        # kk's last entry in F ahead of position j*G
        fseg = fi[g * k * Ls:g * k * Ls + (ns - g * k * Ls if g == groups - 1 else k * Ls)].astype(np.int64)
        frun = fseg // Ls - g * k
        scan_count = {}
        for kk in range(k):
            pos = np.nonzero(frun == kk)[0]
            assert np.array_equal(fseg[pos] - (g * k + kk) * Ls, np.arange(len(pos))), "a run's entries in F out of order"
            scan_count[kk] = np.searchsorted(pos, js * G)
            # boundaries whose scan of 256 entries would miss run kk
            last_before = (np.where(scan_count[kk] > 0, pos[np.maximum(scan_count[kk] - 1, 0)], -1)
                           if len(pos) else np.full(len(js), -1))
            stats["scan_fallbacks"] = stats.get("scan_fallbacks", 0) + int(
                np.sum((js * G - last_before > 256) & (js * G > 256) & (kk != kb)))
            stats["scan_rows"] = stats.get("scan_rows", 0) + int(np.sum(kk != kb))
        for kk in range(k):
            rs = min(kk * L, ng)
            run = keys[gbase + rs:gbase + rs + lens[kk]]
            samp = S[(g * k + kk) * Ls:(g * k + kk) * Ls + ceil_div(lens[kk], B)]
            # earlier runs win ties: keys <= v precede for runs before kb,
            # keys < v for runs after it
            right = kk < kb
            exact = np.where(right, np.searchsorted(run, v, side="right"), np.searchsorted(run, v, side="left"))
            # splitter_kernel: block sample first (m blocks whose first key
            # precedes), then a search inside block m-1, which must bracket
            # the exact count
            m = np.where(right, np.searchsorted(samp, v, side="right"), np.searchsorted(samp, v, side="left"))
            a0 = (m - 1) * B + 1
            a1 = np.minimum(m * B, lens[kk])
            assert np.all(np.where(m == 0, exact == 0, (a0 <= exact) & (exact <= a1)))
            assert np.all(np.where(kk == kb, True, scan_count[kk] == m)), "scan and block-sample search disagree"
            c = np.where(kk == kb, ib, exact)
            desc[1:jg, kk] = c
            desc[jg, kk] = lens[kk]
        doff = desc.sum(axis=1)
        # a last round launched in parts copies out the output prefix before
        # tile T once tiles [0, T) have run (RoundSplit in gms_sort.cuh; the
        # last part copies the rest): an interior tile T starts at or after
        # (T*G - K)*B keys of its group, since of the T*G sampled blocks ahead
        # of boundary T all but the last of each run lie wholly ahead of it
        for j in range(jg):
            assert doff[j] >= max(0, (j * G - k) * B), (j, int(doff[j]), G, k, B)
        for j in range(jg):
            seg_k, seg_i = [], []
            for kk in range(k):
                lo, hi = desc[j, kk], desc[j + 1, kk]
                assert lo <= hi, "boundaries must be monotone per run"
                base = gbase + min(kk * L, ng)
                seg_k.append(keys[base + lo:base + hi])
                seg_i.append(idx[base + lo:base + hi])
            tk = np.concatenate(seg_k)
            ti = np.concatenate(seg_i)
            cnt = len(tk)
            max_tile = max(max_tile, cnt)
            assert cnt <= geo.tile_cap, f"tile of {cnt} keys exceeds {geo.tile_cap} (level {level})"
            assert cnt <= (G + k) * B
            if geo.nt:
                w = windows_per_level([len(x) for x in seg_k], geo.items)
                assert max(w) <= geo.nt, f"tile needs {max(w)} window threads > {geo.nt}"
                stats["max_windows"] = max(stats.get("max_windows", 0), max(w))
            mk, mi = _stable_merge(tk, ti)
            o = gbase + doff[j]
            out_k[o:o + cnt] = mk
            out_i[o:o + cnt] = mi
        assert doff[jg] == ng
    stats.setdefault("max_tile", []).append((level, max_tile))
    stats["tile_launches"] = stats.get("tile_launches", 0) + 1
    return out_k, out_i


def model_sort(keys, geo):
    """Engine::sort: base tiles of CAP, then rounds with L = CAP * K^p."""
    n = len(keys)
    idx = np.arange(n, dtype=np.int64)
    stats = {}
    k = keys.copy()
    for tb in range(0, n, geo.base):
        te = min(n, tb + geo.base)
        k[tb:te], idx[tb:te] = _stable_merge(k[tb:te], idx[tb:te])
    L = geo.base
    rounds = 0
    while L < n:
        k, idx = model_round(k, idx, L, geo, stats)
        L *= geo.k
        rounds += 1
    stats["rounds"] = rounds
    return k, idx, stats
