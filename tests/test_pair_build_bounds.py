"""CPU model of the device's block and key-pair build (gba_kernels.cu:
k_count_pairs, k_block_marks, k_block_lists, k_point_pairs,
k_enumerate_pairs, the radix passes): for ragged batches of synthetic
problems, every index a kernel forms must stay inside its buffer -- codes
inside their problem's Ie x Ie range, block ids below the block count,
which stays below the block lists' capacity, pair positions below the pair
count -- and the numbering must be the host's (blocks in (i, j) order,
every diagonal present)."""
import numpy as np
import pytest

from hs_sfm_gb300 import synthetic

SORT_TILE = 2048   # kSortThreads * kSortPerThread
SCAN_CHUNK = 4096


def point_major(scene):
    """key_img / pt_key_off in the plan's point-major order (images ascending
    within a point)."""
    fm = scene.feature_maps
    order = np.lexsort((fm[:, 0], fm[:, 1]))
    key_img = fm[order, 0].astype(np.int64)
    cnt = np.bincount(fm[:, 1], minlength=scene.number_of_points)
    pt_key_off = np.concatenate([[0], np.cumsum(cnt)])
    return key_img, pt_key_off


def model(scenes):
    # problem records (first image, Ie, first code) and the global arrays
    pinfo, key_img, pt_key_off, pt_prob = [], [], [0], []
    L = ub = img0 = k0 = 0
    for q, s in enumerate(scenes):
        ki, po = point_major(s)
        n = s.number_of_images
        pinfo.append((img0, n, L))
        key_img.append(ki + img0)
        pt_key_off.extend((po[1:] + k0).tolist())
        pt_prob.extend([q] * s.number_of_points)
        L += n * n
        ub += n * (n + 1) // 2
        img0 += n
        k0 += len(ki)
    key_img = np.concatenate(key_img)
    pt_key_off = np.array(pt_key_off)
    P = len(pt_prob)
    # k_count_pairs
    cnt = np.zeros(L, dtype=np.int64)
    for i in range(P):
        x, n, z = pinfo[pt_prob[i]]
        a0, a1 = pt_key_off[i], pt_key_off[i + 1]
        for a in range(a0, a1):
            for c in range(a, a1):
                la, lc = key_img[a] - x, key_img[c] - x
                assert 0 <= la <= lc < n            # images ascending within a point
                e = z + la * n + lc
                assert z <= e < z + n * n and e < L
                cnt[e] += 1
    # k_block_marks + scans + k_block_lists
    mark = np.zeros(L, dtype=np.int64)
    for x, n, z in pinfo:
        for local in range(n * n):
            a, c = divmod(local, n)
            mark[z + local] = 1 if (a == c or (c > a and cnt[z + local] > 0)) else 0
    bid = np.cumsum(mark) - mark
    off = np.cumsum(cnt) - cnt
    nblocks = int(mark.sum())
    total = int(cnt.sum())
    assert nblocks <= ub                            # blk_code / blk_first capacity
    codes = np.nonzero(mark)[0]
    assert np.array_equal(bid[codes], np.arange(nblocks))
    # the host's numbering: per problem, (a, c) lexicographic with a <= c
    host = []
    for x, n, z in pinfo:
        for a in range(n):
            for c in range(a, n):
                if a == c or cnt[z + a * n + c] > 0:
                    host.append(z + a * n + c)
    assert np.array_equal(codes, np.array(host, dtype=np.int64))
    # k_point_pairs + scan, k_enumerate_pairs
    k = np.diff(pt_key_off)
    pp = np.concatenate([[0], np.cumsum(k * (k + 1) // 2)])
    assert pp[-1] == total
    keys = np.empty(total, dtype=np.int64)
    for i in range(P):
        x, n, z = pinfo[pt_prob[i]]
        pos = pp[i]
        a0, a1 = pt_key_off[i], pt_key_off[i + 1]
        for a in range(a0, a1):
            for c in range(a, a1):
                assert 0 <= pos < total
                e = z + (key_img[a] - x) * n + (key_img[c] - x)
                assert mark[e] == 1
                keys[pos] = bid[e]
                pos += 1
        assert pos == pp[i + 1]
    assert keys.min(initial=0) >= 0 and (total == 0 or keys.max() < nblocks)
    # radix passes: digits of bits(nblocks), histogram of 256 x tiles entries
    bits = 1
    while bits < 31 and (1 << bits) < nblocks:
        bits += 1
    passes = (bits + 7) // 8
    ntiles = (total + SORT_TILE - 1) // SORT_TILE
    assert keys.max(initial=0) < (1 << (8 * passes))
    hist = 256 * max(ntiles, 1)
    assert (hist + SCAN_CHUNK - 1) // SCAN_CHUNK >= 1
    # the stable sort by block id gives each block's pairs in point order
    order = np.argsort(keys, kind="stable")
    firsts = off[codes]
    sorted_keys = keys[order]
    for b in range(nblocks):
        seg = sorted_keys[firsts[b]:firsts[b] + cnt[codes[b]]]
        assert np.all(seg == b)
    return nblocks, total


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_ragged_batches_stay_in_bounds(seed):
    rng = np.random.default_rng(seed)
    scenes = []
    for _ in range(int(rng.integers(1, 5))):
        ni = int(rng.integers(1, 9))
        npts = int(rng.integers(0, 60))
        scenes.append(synthetic.ring_scene(num_images=ni, num_points=max(npts, 1),
                                           obs_range=(1, min(ni, 5)), seed=int(rng.integers(1 << 30))))
    nb, total = model(scenes)
    assert nb >= sum(s.number_of_images for s in scenes)   # every diagonal block


def test_single_grid_problem():
    s = synthetic.grid_scene(num_images=12, num_points=300, seed=3)
    nb, total = model([s])
    assert total > 0 and nb >= 12
