"""The index arithmetic of the rows-to-columns sort (ac-dc_gb300/csrc/transpose.cu),
restated step by step on the CPU: tiles of 4096 entries, chunks of 256 with
8 warps of 32 lanes, digit counts per (digit, tile) scanned digit-major, and
each entry placed at its digit's base + the counts of earlier warps + its rank
among equal digits of its own warp.  Every position must fall inside the
arrays, none twice, and the result must equal a stable sort by column (each
column's entries in row order), for one to three 8-bit passes."""
import numpy as np
import pytest

TILE, THREADS, WARPS = 4096, 256, 8


def model(m, n, row_ptr, col, val):
    nnz = int(row_ptr[m])
    rows_of = np.repeat(np.arange(m), np.diff(row_ptr))
    col = np.where((col < 0) | (col >= n), 0, col)  # flagged and sorted as column 0
    col_ptr = np.concatenate([[0], np.cumsum(np.bincount(col, minlength=n))])
    tiles = (nnz + TILE - 1) // TILE
    bits = 1
    while bits < 31 and (1 << bits) < n:
        bits += 1
    keys, rows, vals = col.copy(), rows_of.copy(), val.copy()
    for shift in range(0, 8 * ((bits + 7) // 8), 8):
        digit = (keys >> shift) & 255
        hist = np.zeros((256, tiles), np.int64)
        for t in range(tiles):
            hist[:, t] = np.bincount(digit[t * TILE:(t + 1) * TILE], minlength=256)
        offs = np.concatenate([[0], np.cumsum(hist.ravel())])  # digit-major
        out = np.full(nnz, -1)
        for t in range(tiles):
            base = offs[np.arange(256) * tiles + t].copy()
            end = min((t + 1) * TILE, nnz)
            for c in range(t * TILE, end, THREADS):
                d = np.full(THREADS, -1)
                k = min(THREADS, end - c)
                d[:k] = digit[c:c + k]
                wcnt = np.zeros((WARPS, 256), np.int64)
                pos = np.zeros(THREADS, np.int64)
                for w in range(WARPS):
                    dw = d[32 * w:32 * (w + 1)]
                    for lane in range(32):
                        if dw[lane] < 0:
                            continue
                        rank = int(np.sum(dw[:lane] == dw[lane]))  # __match_any_sync rank
                        pos[32 * w + lane] = rank
                        if rank == 0:
                            wcnt[w, dw[lane]] = int(np.sum(dw == dw[lane]))
                for th in range(k):
                    w = th >> 5
                    p = base[d[th]] + pos[th] + wcnt[:w, d[th]].sum()
                    assert 0 <= p < nnz and out[p] == -1
                    out[p] = c + th
                base += wcnt.sum(axis=0)
        assert (out >= 0).all()
        keys, rows, vals = keys[out], rows[out], vals[out]
    return col_ptr, rows, vals


@pytest.mark.parametrize("m,n,nnz", [(1, 1, 1), (5, 3, 0), (40, 300, 600), (120, 70000, 4500),
                                     (2500, 2, 4300)])
def test_radix_transpose_model_is_a_stable_column_sort(m, n, nnz):
    rng = np.random.default_rng(m + n + nnz)
    lens = rng.multinomial(nnz, np.ones(m) / m)
    row_ptr = np.concatenate([[0], np.cumsum(lens)])
    col = (np.concatenate([np.sort(rng.choice(n, size=k, replace=k > n)) for k in lens])
           if nnz else np.zeros(0, np.int64)).astype(np.int64)
    val = rng.normal(size=nnz)
    cp, r, v = model(m, n, row_ptr, col, val)
    rows_of = np.repeat(np.arange(m), lens)
    order = np.lexsort((rows_of, col))  # by column, then row
    assert np.array_equal(cp, np.concatenate([[0], np.cumsum(np.bincount(col, minlength=n))]))
    assert np.array_equal(r, rows_of[order]) and np.array_equal(v, val[order])
