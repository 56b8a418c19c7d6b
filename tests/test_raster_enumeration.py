"""Host restatements of the raster stage's index bookkeeping (raster_kernels.cu, raster_tile),
checked on random inputs: they decide which (record, row, column) every lane visits, so an error
would drop or repeat pixels rather than change arithmetic.

* span walk: a batch's spans (pixel offset | record << 16 | row << 24 | first column << 28) tile
  the pixel range [0, P); each warp walks a contiguous range in chunks of 32, finds the span of
  every lane from a window of the next 32 span starts (a bit mask of the starts falling inside
  the chunk, the lane's rank in it), and advances by the number of spans starting at or before
  the next chunk.  Every pixel must be visited exactly once with its own span's fields.
* row jobs: a warp's 32 records own consecutive runs of (record, row) jobs (an inclusive scan of
  their row counts); the owner of job j is the last lane whose first job is at or before j,
  found by a 5-step search over shuffled prefixes.  Records without rows must never be chosen.
* coalesced single-launch scan: warp w owns 1024 consecutive tiles as 32 rows of 32; rows are
  scanned across the lanes in order, then the warp totals; the result must equal the exclusive
  prefix sum."""
import numpy as np


def popc(x):
    return bin(x & 0xFFFFFFFF).count("1")


def span_walk(spans, P, NT=256):
    NW, NSP = NT // 32, len(spans)
    per = (P + NT - 1) // NT * 32
    seen = {}
    for wid in range(NW):
        pb, pe = wid * per, min(P, wid * per + per)
        if pb >= pe:
            continue
        s0, hi = 0, NSP - 1
        while s0 < hi:
            mid = (s0 + hi + 1) >> 1
            if (spans[mid] & 0xFFFF) <= pb:
                s0 = mid
            else:
                hi = mid - 1
        w0 = spans[s0]
        for p0 in range(pb, pe, 32):
            wl = [spans[s0 + 1 + l] if s0 + 1 + l < NSP else 0 for l in range(32)]
            d = [((spans[s0 + 1 + l] & 0xFFFF) - p0) & 0xFFFFFFFF if s0 + 1 + l < NSP else 0xFFFFFFFF
                 for l in range(32)]
            M = 0
            for x in d:
                if x < 32:
                    M |= 1 << x
            adv = sum(1 for x in d if x <= 32)
            for lane in range(32):
                rank = popc(M & ((2 << lane) - 1))
                sw = wl[rank - 1] if rank else w0
                p = p0 + lane
                if p >= pe:
                    continue
                assert p not in seen
                seen[p] = ((sw >> 16) & 0xFF, (sw >> 24) & 15, (sw >> 28) + (p - (sw & 0xFFFF)))
            if adv:
                w0 = wl[adv - 1]
            s0 += adv
    return seen


def test_span_walk_visits_every_pixel_once():
    rng = np.random.default_rng(3)
    for _ in range(300):
        spans, truth, p = [], {}, 0
        for r in range(int(rng.integers(1, 257))):
            for row in range(16):
                if rng.uniform() < 0.3 and len(spans) < 2048:
                    lo = int(rng.integers(0, 16))
                    hi = int(rng.integers(lo, 16)) if rng.uniform() < 0.5 else min(15, lo + int(rng.integers(0, 3)))
                    spans.append(p | (r << 16) | (row << 24) | (lo << 28))
                    for x in range(lo, hi + 1):
                        truth[p] = (r, row, x)
                        p += 1
        if spans:
            assert span_walk(spans, p) == truth


def test_row_job_owner_search():
    rng = np.random.default_rng(4)
    for _ in range(2000):
        rows = rng.integers(0, 17, 32) * (rng.uniform(size=32) < 0.8)
        incl = np.cumsum(rows)
        pre = incl - rows
        J = int(incl[-1])
        for j in range(J):
            k = 0
            for step in (16, 8, 4, 2, 1):
                if pre[k + step] <= j:
                    k += step
            assert rows[k] > 0 and pre[k] <= j < pre[k] + rows[k]


def test_single_launch_scan_layout():
    rng = np.random.default_rng(5)
    for T in (1, 31, 1024, 1025, 8160, 32400, 32768):
        cnt = rng.integers(0, 50, T)
        padded = np.zeros(32 * 1024, np.int64)
        padded[:T] = cnt
        blocks = padded.reshape(32, 32, 32)  # [warp][row][lane]
        within = np.cumsum(blocks.reshape(32, -1), 1).reshape(32, 32, 32) - blocks
        warp_tot = blocks.reshape(32, -1).sum(1)
        out = (within + (np.cumsum(warp_tot) - warp_tot)[:, None, None]).reshape(-1)[:T]
        assert (out == np.concatenate([[0], np.cumsum(cnt)[:-1]])).all()
