"""The plain kernel's row-buffer bound, on a model of its walk.

The shared-memory merge (pairs_kernel, VAR 5) advances the row on every step
whose row time is not later than the column time, and a warp runs
`L_row + max L_col - 1` steps rounded up to blocks of U.  A lane whose pair is
done therefore keeps advancing its row; the kernel pulls the row address back
to the row's last element at every block start, so the row buffer needs only
U sentinel copies past the row.  This models that walk step by step (times
staged as the kernel stages them: clamped to TMAX, NaN included, last element
TMAX) and checks, for sorted and for arbitrary rows, that no read passes
`L_row - 1 + U` and that the pull-back leaves every rectangle as it was.
"""
import numpy as np

TMAX = np.float32(np.finfo(np.float32).max)
U = 8


def staged(t):
    """Segment layout times: element k ends at t[k+1]; the last at TMAX."""
    tn = np.empty(len(t), np.float32)
    tn[:-1] = np.fmin(t[1:], TMAX)  # fmin: NaN -> TMAX, as clamp_time
    tn[-1] = TMAX
    return tn


def walk(row_tn, row_pad, col_tn, steps, pull_back):
    """Rectangles (t_prev, t_next, row index, col index) and the largest row index read."""
    rlen = len(row_tn)
    rt = np.concatenate([row_tn, np.full(row_pad, TMAX, np.float32)])
    fi, gi, t = 0, 0, np.float32(0)
    rects, max_read = [], 0
    nblk = (steps + U - 1) // U
    for _ in range(nblk):
        if pull_back:
            fi = min(fi, rlen - 1)
        for _ in range(U):
            ft, gt = rt[fi], col_tn[gi]
            tn = min(ft, gt)
            rects.append((t, tn, min(fi, rlen - 1), gi))
            t = tn
            if ft <= gt:
                fi += 1
                max_read = max(max_read, fi)
                assert fi < len(rt), "row read past the buffer"
            else:
                gi += 1
                assert gi < len(col_tn), "column advanced past its sentinel"
    return rects, max_read


def test_pull_back_bounds_row_reads_and_keeps_rectangles():
    rng = np.random.default_rng(0)
    for case in range(400):
        rlen = int(rng.integers(1, 60))
        clens = rng.integers(1, 80, size=4)
        maxlc = int(clens.max())
        kind = case % 3
        if kind == 0:  # sorted, as the PCF contract has it
            row_t = np.concatenate([[0], np.cumsum(rng.exponential(1, rlen - 1))]).astype(np.float32)
        elif kind == 1:  # ties and repeats
            row_t = np.concatenate([[0], np.cumsum(rng.integers(0, 2, rlen - 1))]).astype(np.float32)
        else:  # arbitrary data, NaN and inf included
            row_t = rng.normal(0, 5, rlen).astype(np.float32)
            row_t[rng.random(rlen) < 0.1] = np.nan
            row_t[rng.random(rlen) < 0.1] = np.inf
        row_tn = staged(row_t)
        steps = rlen + maxlc - 1
        for cl in clens:
            col_t = np.concatenate([[0], np.cumsum(rng.exponential(1, int(cl) - 1))]).astype(np.float32)
            col_tn = staged(col_t)
            full, _ = walk(row_tn, maxlc + U, col_tn, steps, pull_back=False)
            short, max_read = walk(row_tn, U, col_tn, steps, pull_back=True)
            assert max_read <= rlen - 1 + U
            # the same rectangles: widths, and the values in force (row index
            # past the end reads a sentinel copy of the last element)
            assert [(a, b, r, g) for a, b, r, g in full] == [(a, b, r, g) for a, b, r, g in short]
