"""CPU model of the dense-Cholesky launches of libgba.so: for batches of
problems of uneven size, every S / b / Linv element a kernel touches must
lie inside that problem's own region.  The model restates each kernel's
grid and early-exit guards (hs_sfm_gb300/csrc/gba_kernels.cu: k_chol_step for
k = -1 .. nt-2 with its redundant per-column diagonal factorization,
the cluster backward solve k_chol_solve, k_assemble_S)."""
import math

import numpy as np
import pytest

TILE = 32


def rows(n, t):
    return min(TILE, n - TILE * t)


def decode(lin):
    ti = int((math.sqrt(8.0 * lin + 1.0) - 1.0) * 0.5)
    while (ti + 1) * (ti + 2) // 2 <= lin:
        ti += 1
    while ti * (ti + 1) // 2 > lin:
        ti -= 1
    return ti, lin - ti * (ti + 1) // 2


class Batch:
    def __init__(self, images):
        self.I = list(images)
        self.n = [6 * i for i in images]
        self.nt = [(n + TILE - 1) // TILE for n in self.n]
        self.s_off = np.concatenate([[0], np.cumsum([n * n for n in self.n])]).tolist()
        self.img_begin = np.concatenate([[0], np.cumsum(images)]).tolist()
        self.max_nt = max(self.nt)
        self.max_n = max(self.n)
        self.B = len(images)

    def check_S(self, p, r0, nr, c0, nc):
        n = self.n[p]
        assert nr >= 0 and nc >= 0
        if nr == 0 or nc == 0:
            return
        assert 0 <= r0 and r0 + nr <= n and 0 <= c0 and c0 + nc <= n, (p, r0, nr, c0, nc, n)
        lo = self.s_off[p] + r0 * n + c0
        hi = self.s_off[p] + (r0 + nr - 1) * n + c0 + nc - 1
        assert self.s_off[p] <= lo and hi < self.s_off[p + 1]

    def check_b(self, p, e0, ne):
        lo = 6 * self.img_begin[p] + e0
        assert 0 <= e0 and e0 + ne <= self.n[p], (p, e0, ne)
        assert 6 * self.img_begin[p] <= lo and lo + ne <= 6 * self.img_begin[p + 1]

    def check_linv(self, p, k):
        assert 0 <= k < self.max_nt
        assert 0 <= p * self.max_nt + k < self.B * self.max_nt

    def diag(self, p, k):
        m = rows(self.n[p], k)
        self.check_S(p, TILE * k, m, TILE * k, m)
        self.check_linv(p, k)
        self.check_b(p, TILE * k, m)

    def step_tile(self, p, k, i, j):
        n, c = self.n[p], k + 1
        mi, mj = rows(n, i), rows(n, j)
        assert c <= j <= i < self.nt[p]
        self.check_S(p, TILE * i, mi, TILE * j, mj)            # own tile
        if k >= 0:
            assert k <= self.nt[p] - 2                         # tile k is full
            self.check_S(p, TILE * i, mi, TILE * k, rows(n, k))
            self.check_S(p, TILE * j, mj, TILE * k, rows(n, k))
            self.check_b(p, TILE * k, TILE)                    # y_k
        if j == c:
            self.check_S(p, TILE * c, rows(n, c), TILE * c, rows(n, c))  # diagonal tile
            self.check_b(p, TILE * i, mi)
            if i == c:
                self.check_linv(p, c)

    def solve(self, p, ranks=8, warps=8):
        """k_chol_solve: rank q owns tile rows t = q (mod ranks), local row
        lt = t // ranks; warp w owns the local rows lt = w (mod warps).  The
        dynamic shared memory holds max_nt mbarriers, max_nt delta slots of
        TILE entries and ceil(max_nt / ranks) rows of y."""
        n, nt, mt = self.n[p], self.nt[p], self.max_nt
        slots, y_rows = mt, (mt + ranks - 1) // ranks
        owner = {}
        for q in range(ranks):
            nown = (nt - q + ranks - 1) // ranks if nt > q else 0
            assert nown <= y_rows
            for lt in range(nown):                    # ys load
                t = q + ranks * lt
                self.check_b(p, TILE * t, rows(n, t))
            for w in range(warps):
                mine = [lt for lt in range(w, nown, warps)]
                for lt in mine:                       # delta of the warp's rows
                    t = q + ranks * lt
                    assert t not in owner
                    owner[t] = (q, w)
                    self.check_linv(p, t)
                    self.check_b(p, TILE * t, rows(n, t))
                for j in range(nt - 1, -1, -1):
                    assert j < slots                  # slot j and mbarrier j
                    below = [lt for lt in mine if q + ranks * lt < j]
                    for lt in below:                  # L_ji^T delta_j into row i
                        i = q + ranks * lt
                        assert lt < y_rows and i < j and i <= nt - 2   # tile i is full
                        self.check_S(p, TILE * j, rows(n, j), TILE * i, TILE)
        assert sorted(owner) == list(range(nt))       # every step has one owner

    def run(self):
        touched = 0
        for bx in range(self.max_nt):                 # k_chol_step, k = -1
            for p in range(self.B):
                if bx >= self.nt[p]:
                    continue
                self.step_tile(p, -1, bx, 0)
                touched += 1
        for k in range(self.max_nt - 1):              # k_chol_step, k >= 0
            Tg = self.max_nt - k - 1
            for lin in range(Tg * (Tg + 1) // 2):
                for p in range(self.B):
                    Tn = self.nt[p] - (k + 1)
                    if Tn <= 0 or lin >= Tn * (Tn + 1) // 2:
                        continue
                    ti, tj = decode(lin)
                    self.step_tile(p, k, k + 1 + ti, k + 1 + tj)
                    touched += 1
        for p in range(self.B):                       # k_chol_solve, cluster per problem
            self.solve(p)
        # k_assemble_S: thread (row, col) of the lower triangle
        for p in range(self.B):
            n, I = self.n[p], self.I[p]
            assert (self.max_n * self.max_n + 255) // 256 * 256 >= n * n
            if n:
                self.check_S(p, 0, n, 0, n)
                self.check_b(p, 0, n)
                assert (n - 1) // 6 < I
        return touched


@pytest.mark.parametrize("images", [
    [14, 32], [15, 39], [39, 15], [5, 40, 5, 40], [1, 2, 3], [200], [40] * 3,
    [14, 32, 15, 34, 34, 39],
])
def test_cholesky_accesses_stay_inside_each_problem(images):
    Batch(images).run()


def test_random_batches():
    rng = np.random.default_rng(0)
    for _ in range(40):
        Batch(list(rng.integers(1, 48, size=rng.integers(1, 9)))).run()


def test_decode_covers_the_lower_triangle():
    for T in range(1, 40):
        seen = {decode(lin) for lin in range(T * (T + 1) // 2)}
        assert seen == {(i, j) for i in range(T) for j in range(i + 1)}
