"""The single-LP engine's matrix layout (host plan), checked on the CPU.

The plan code of sovereign-solver_gb300/csrc/engine_impl.cuh (the SLAB choice
by sampled sector counts, the bins, slice offsets, unit descriptors, tickets,
epilogue slots and block shares) runs through a host-only helper
(tests/plan_dump.cu, built here with nvcc); this test then replays the pass
kernels' traversal of the plan (engine.cuh visit_bins: SLICED slice pairs,
WARP row pairs, SEGMENT pairs with per-row tickets, SLAB units with per-slice
tickets) in NumPy, with the units taken in a shuffled order, and checks every
index against its array, one epilogue per row, tickets back at zero, every
slot used once and the row sums against a direct CSR product."""

import os
import shutil
import struct
import subprocess

import numpy as np
import pytest
import scipy.sparse as sp

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
KWARPS, KSEG, KSLAB = 8, 512, 32
SLICED, WARP, SEGMENT, SLAB = 0, 1, 2, 3


@pytest.fixture(scope="module")
def plan_tool(tmp_path_factory):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    out = str(tmp_path_factory.mktemp("plan") / "plan_dump")
    cmd = [nvcc, "-std=c++17", "-O1", "-gencode", "arch=compute_103a,code=sm_103a",
           f"-I{os.path.join(ROOT, 'include')}", f"-I{os.path.join(ROOT, 'sovereign-solver_gb300', 'csrc')}",
           os.path.join(HERE, "plan_dump.cu"), "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    return out


def run_plan(tool, tmp, ptr, idx, kind, n, inv_col, cap, cols=False):
    m = len(ptr) - 1
    fin, fout = os.path.join(tmp, "in.bin"), os.path.join(tmp, "out.bin")
    with open(fin, "wb") as f:
        f.write(struct.pack("<iiq", m, n, int(ptr[-1])))
        f.write(np.asarray(ptr, np.int32).tobytes())
        f.write(np.asarray(idx, np.int32).tobytes())
        f.write(np.asarray(kind, np.int8).tobytes())
        f.write(np.asarray(inv_col, np.int32).tobytes())
    subprocess.run([tool, fin, fout, str(cap)] + (["cols"] if cols else []), check=True)
    arrs = []
    with open(fout, "rb") as f:
        for _ in range(7):
            (cnt,) = struct.unpack("<q", f.read(8))
            arrs.append(np.frombuffer(f.read(4 * cnt), np.int32).copy())
    slab, perm, fptr, soff, unit, bins, tail = arrs
    return dict(slab=slab, perm=perm, fptr=fptr, soff=soff, unit=unit.reshape(-1, 8),
                bins=bins[2:].reshape(bins[0], 12), total_blocks=int(bins[1]),
                total=int(tail[0]), ntickets=int(tail[1]), nslots=int(tail[2]), nslab=int(tail[3]))


def check_plan(tool, tmp, ptr, idx, kind, n, inv_col, cap=760, seed=0, cols=False):
    """Replay the traversal; returns the plan's bins as (mode, kind, rows)."""
    rng = np.random.default_rng(seed)
    ptr = np.asarray(ptr, np.int64)
    idx = np.asarray(idx, np.int64)
    inv_col = np.asarray(inv_col)
    m = len(ptr) - 1
    P = run_plan(tool, tmp, ptr, idx, kind, n, inv_col, cap, cols)
    perm, fptr, soff, unit, B, total = P["perm"], P["fptr"], P["soff"], P["unit"], P["bins"], P["total"]
    assert sorted(perm.tolist()) == list(range(m))
    assert P["total_blocks"] <= cap and B[:, 5].sum() == P["total_blocks"]
    vals = rng.standard_normal(len(idx))
    # internal CSR (rows in plan order, columns renumbered) and the final layout
    tptr = np.zeros(m + 1, np.int64)
    for r in range(m):
        tptr[r + 1] = tptr[r] + ptr[perm[r] + 1] - ptr[perm[r]]
    tidx = np.concatenate([inv_col[idx[ptr[o]:ptr[o + 1]]] for o in perm]) if m else np.zeros(0, np.int64)
    tval = np.concatenate([vals[ptr[o]:ptr[o + 1]] for o in perm]) if m else np.zeros(0)
    fidx = np.full(max(total, 1), -1, np.int64)
    fval = np.full(max(total, 1), np.nan)
    for (beg, end, mode, _k, _bb, _nb, units, aux, _a2, slice0, part0, _s0) in B:
        if mode == SEGMENT:
            # a row's last segment acquires by a load of its ticket in bins of at most
            # 4096 rows, by a fence in larger ones (engine.cuh kSegLoadAcquireRows)
            assert part0 == (1 if end - beg <= 4096 else 0)
        if mode in (SLICED, SLAB):
            first, nsl = (aux, units) if mode == SLICED else (slice0, (end - beg + 31) // 32)
            for s in range(nsl):
                off, L = soff[first + s], (soff[first + s + 1] - soff[first + s]) >> 5
                if mode == SLICED and part0 > 0:
                    assert off == slice0 + s * 32 * part0 and L == part0
                for lane in range(32):
                    r = beg + 32 * s + lane
                    ln = tptr[r + 1] - tptr[r] if r < end else 0
                    assert ln <= L
                    for k in range(L):
                        fidx[off + 32 * k + lane] = tidx[tptr[r] + k] if k < ln else 0
                        fval[off + 32 * k + lane] = tval[tptr[r] + k] if k < ln else 0.0
        else:
            for r in range(beg, end):
                d, ln = fptr[r], tptr[r + 1] - tptr[r]
                fidx[d:d + ln] = tidx[tptr[r]:tptr[r + 1]]
                fval[d:d + ln] = tval[tptr[r]:tptr[r + 1]]
    x = rng.standard_normal(n)
    want = np.array([(tval[tptr[r]:tptr[r + 1]] * x[tidx[tptr[r]:tptr[r + 1]]]).sum() for r in range(m)])

    def gat(p):
        assert 0 <= p < total
        assert 0 <= fidx[p] < n
        return fval[p] * x[fidx[p]]

    got = np.full(m, np.nan)
    hits = np.zeros(m, int)
    tickets = np.zeros(max(P["ntickets"], 1), int)
    slots = np.zeros(max(P["nslots"], 1), int)
    segpart, slabpart = {}, {}
    items = []
    for bi, b in enumerate(B):
        mode, bb, nbk, units = b[2], b[4], b[5], b[6]
        stride = nbk * KWARPS
        for blk in range(bb, bb + nbk):
            for w in range(KWARPS):
                u = (blk - bb) * KWARPS + w
                while u < units:
                    items.append((bi, u, u + stride))
                    u += stride if mode == SLAB else 2 * stride
    for it in rng.permutation(len(items)):
        bi, u0, u1 = items[it]
        beg, end, mode, _k, _bb, _nb, units, aux, aux2, slice0, part0, slot0 = B[bi]
        pair = [u0] + ([u1] if u1 < units else [])
        if mode == SLICED:
            for s in pair:
                off, L = soff[aux + s], (soff[aux + s + 1] - soff[aux + s]) >> 5
                for lane in range(32):
                    r = beg + 32 * s + lane
                    acc = sum(gat(off + lane + 32 * k) for k in range(L))
                    if r < end:
                        got[r] = acc
                        hits[r] += 1
        elif mode == WARP:
            for u in pair:
                r = beg + u
                got[r] = sum(gat(p) for p in range(fptr[r], fptr[r + 1]))
                hits[r] += 1
        elif mode == SEGMENT:
            for u in pair:
                gs = aux + u
                s_, t_, r, nseg, kk = unit[gs][:5]
                assert beg <= r < end and s_ == fptr[r] + kk * KSEG and t_ == min(fptr[r + 1], s_ + KSEG)
                assert nseg == (fptr[r + 1] - fptr[r] + KSEG - 1) // KSEG
                segpart[gs] = sum(gat(p) for p in range(s_, t_))
                tk = aux2 + (r - beg)
                tickets[tk] += 1
                if tickets[tk] != nseg:
                    continue
                tickets[tk] = 0
                got[r] = sum(segpart[gs - kk + q] for q in range(nseg))
                hits[r] += 1
                slots[slot0 + (r - beg)] += 1
        else:
            gu = aux + u0
            off, L, s, c = unit[gu][:4]
            assert soff[slice0 + s] == off and (soff[slice0 + s + 1] - off) >> 5 == L
            k0, k1 = c * KSLAB, min(L, c * KSLAB + KSLAB)
            acc = np.array([sum(gat(off + 32 * k + lane) for k in range(k0, k1)) for lane in range(32)])
            nun = (L + KSLAB - 1) // KSLAB
            if nun > 1:
                pu = part0 + u0                          # a SLAB bin's units in the SLAB partials
                assert 0 <= pu < P["nslab"]
                slabpart[pu] = acc
                tickets[aux2 + s] += 1
                if tickets[aux2 + s] != nun:
                    continue
                tickets[aux2 + s] = 0
                for w in range(nun):
                    assert unit[gu - c + w][2] == s and unit[gu - c + w][3] == w
                acc = sum(slabpart[pu - c + w] for w in range(nun))
            for lane in range(32):
                r = beg + 32 * s + lane
                if r < end:
                    got[r] = acc[lane]
                    hits[r] += 1
            slots[slot0 + s] += 1
    assert (hits == 1).all()
    assert (tickets == 0).all()
    assert (slots[:P["nslots"]] == 1).all()
    np.testing.assert_allclose(got, want, rtol=1e-12, atol=1e-12)
    return [(int(b[2]), int(b[3]), int(b[1] - b[0])) for b in B]


def transport(S, D):
    rows = [np.arange(i * D, (i + 1) * D) for i in range(S)] + [np.arange(S) * D + j for j in range(D)]
    return np.cumsum([0] + [len(r) for r in rows]), np.concatenate(rows), [1] * S + [0] * D, S * D


def test_transportation_demand_rows_take_slab(plan_tool, tmp_path):
    ptr, idx, kind, n = transport(40, 70)
    bins = check_plan(plan_tool, str(tmp_path), ptr, idx, kind, n, np.arange(n))
    # the 70 demand rows (stride-40 columns): two full groups of 32 in SLAB; the
    # 40 supply rows (contiguous columns) stay CSR
    assert (SLAB, 0, 64) in bins and (WARP, 1, 40) in bins


def test_small_block_cap(plan_tool, tmp_path):
    ptr, idx, kind, n = transport(33, 45)
    check_plan(plan_tool, str(tmp_path), ptr, idx, kind, n, np.arange(n), cap=7)


def test_ragged_rows_every_schedule(plan_tool, tmp_path):
    rng = np.random.default_rng(1)
    rows = [r + 50 * np.arange(int(rng.integers(40, 90))) for r in range(100)]          # shifted, ragged
    rows += [np.sort(rng.choice(6000, int(rng.integers(33, 1500)), replace=False)) for _ in range(50)]
    rows += [np.sort(rng.choice(6000, int(rng.integers(1, 33)), replace=False)) for _ in range(70)]
    ptr = np.cumsum([0] + [len(r) for r in rows])
    idx = np.concatenate(rows)
    bins = check_plan(plan_tool, str(tmp_path), ptr, idx, list(rng.integers(0, 2, len(rows))), 6000,
                      np.arange(6000))
    assert {b[0] for b in bins} == {SLICED, WARP, SEGMENT, SLAB}
    check_plan(plan_tool, str(tmp_path), ptr, idx, [0] * len(rows), 6000, np.arange(6000))
    # a column permutation destroys the shifted pattern: no SLAB rows
    bins = check_plan(plan_tool, str(tmp_path), ptr, idx, [0] * len(rows), 6000, rng.permutation(6000))
    assert SLAB not in {b[0] for b in bins}


def test_long_shifted_rows_multi_unit_slices(plan_tool, tmp_path):
    rows = [r + 300 * np.arange(700) for r in range(45)] + [np.arange(1300) + 7 * r for r in range(5)]
    ptr = np.cumsum([0] + [len(r) for r in rows])
    n = 300 * 700 + 64
    bins = check_plan(plan_tool, str(tmp_path), ptr, np.concatenate(rows), [0] * len(rows), n, np.arange(n))
    assert (SLAB, 0, 32) in bins


def test_uniform_short_rows_compute_offsets(plan_tool, tmp_path):
    rows = [np.array([i % 50, 50 + (i % 70)]) for i in range(300)]
    ptr = np.cumsum([0] + [len(r) for r in rows])
    P = run_plan(plan_tool, str(tmp_path), ptr, np.concatenate(rows), [0] * 300, 120, np.arange(120), 760)
    assert P["bins"][0][2] == SLICED and P["bins"][0][10] == 2
    check_plan(plan_tool, str(tmp_path), ptr, np.concatenate(rows), [0] * 300, 120, np.arange(120))


@pytest.mark.parametrize("cap", [8, 9, 11, 12, 13])
def test_block_shares_fit_the_cap(plan_tool, tmp_path, cap):
    """Eight bins (four schedules x two row kinds) sharing fewer blocks than
    they need (14 blocks): the proportional shares add up to the cap, never past
    it (each block past one resident wave waits for a free slot)."""
    rng = np.random.default_rng(1)
    rows = [r + 50 * np.arange(int(rng.integers(40, 90))) for r in range(100)]
    rows += [np.sort(rng.choice(6000, int(rng.integers(33, 1500)), replace=False)) for _ in range(50)]
    rows += [np.sort(rng.choice(6000, int(rng.integers(1, 33)), replace=False)) for _ in range(70)]
    ptr = np.cumsum([0] + [len(r) for r in rows])
    idx = np.concatenate(rows)
    kind = list(rng.integers(0, 2, len(rows)))
    P = run_plan(plan_tool, str(tmp_path), ptr, idx, kind, 6000, np.arange(6000), cap)
    assert len(P["bins"]) == 8 and P["total_blocks"] == cap
    check_plan(plan_tool, str(tmp_path), ptr, idx, kind, 6000, np.arange(6000), cap=cap)


@pytest.mark.parametrize("cap", [760, 16])
def test_power_law_rows(plan_tool, tmp_path, cap):
    """A small power-law LP (Zipf(1.5) row lengths clipped to [2, 3000], uniform
    random columns, the shape of the 1M x 2M roofline workload): rows in every
    CSR schedule, ragged SEGMENT rows of up to six segments, in one wave and
    with proportional shares of a small cap."""
    rng = np.random.default_rng(5)
    m, n = 1500, 4000
    lens = np.clip(rng.zipf(1.5, m), 2, 3000)
    rows = [np.sort(rng.choice(n, int(k), replace=False)) for k in lens]
    ptr = np.cumsum([0] + [len(r) for r in rows])
    bins = check_plan(plan_tool, str(tmp_path), ptr, np.concatenate(rows), [0] * m, n, np.arange(n), cap=cap)
    assert {b[0] for b in bins} == {SLICED, WARP, SEGMENT}


@pytest.mark.parametrize("cap", [760, 11])
def test_column_plans(plan_tool, tmp_path, cap):
    """The column plan as the engine makes it (one kind, no SLAB choice), on
    the columns of a transportation LP (all of length 2: one SLICED bin with
    computed slice offsets) and of a power-law LP (every CSR schedule)."""
    ptr, idx, kind, n = transport(30, 50)
    M = sp.csr_matrix((np.ones(len(idx)), idx, ptr), shape=(len(ptr) - 1, n)).tocsc()
    bins = check_plan(plan_tool, str(tmp_path), M.indptr, M.indices, [0] * n, M.shape[0],
                      np.arange(M.shape[0]), cap=cap, cols=True)
    assert bins == [(SLICED, 0, n)]
    rng = np.random.default_rng(6)
    m, n = 600, 900
    rows = [np.sort(rng.choice(n, int(k), replace=False)) for k in np.clip(rng.zipf(1.3, m), 1, 900)]
    ptr = np.cumsum([0] + [len(r) for r in rows])
    M = sp.csr_matrix((np.ones(ptr[-1]), np.concatenate(rows), ptr), shape=(m, n)).T.tocsr()
    bins = check_plan(plan_tool, str(tmp_path), M.indptr, M.indices, [0] * n, m, np.arange(m), cap=cap, cols=True)
    assert {b[0] for b in bins} <= {SLICED, WARP, SEGMENT} and {b[1] for b in bins} == {0}


def test_segment_bin_acquire_choice(plan_tool, tmp_path):
    """SEGMENT rows: a bin of at most 4096 rows has its rows' last segments acquire
    by a load of the row ticket (part0 = 1), a larger bin by a fence (part0 = 0);
    the plan only, without the traversal replay (2.2M entries)."""
    rng = np.random.default_rng(11)
    n = 20000
    for m, want in ((4096, 1), (4200, 0)):
        lens = np.full(m, 520)                       # two segments per row, random columns
        idx = np.concatenate([rng.choice(n, 520, replace=False) for _ in range(m)])
        ptr = np.concatenate([[0], np.cumsum(lens)])
        P = run_plan(plan_tool, str(tmp_path), ptr, idx, [0] * m, n, np.arange(n), 760)
        seg = [b for b in P["bins"] if b[2] == SEGMENT]
        assert len(seg) == 1 and seg[0][1] - seg[0][0] == m
        assert seg[0][10] == want


def test_many_slab_groups(plan_tool, tmp_path):
    """600 demand rows of 40 entries (stride-40 columns): 19 groups of up to 32
    rows, scored on two host-pool threads (the SLAB choice runs its groups in
    parallel from 16 groups on); every group takes SLAB and the traversal replay
    checks the layout."""
    ptr, idx, kind, n = transport(40, 600)
    bins = check_plan(plan_tool, str(tmp_path), ptr, idx, kind, n, np.arange(n))
    assert (SLAB, 0, 600) in bins and (SEGMENT, 1, 40) in bins
