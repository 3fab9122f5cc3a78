"""Load-balanced search and race-and-resolve on the GPU against the oracle.

LBS must be bit-exact (int32 scan, owners, total) against the golden vectors of
the reference's examples/load_balanced_search/lbs.cu and against
oracle/gu_oracle.c on larger inputs, including the per-vertex degree array of
the 2048 x 2048 grid (4,194,304 counts).
"""
import numpy as np
import pytest

import gu
import oracle
from conftest import golden_names, load_golden

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def run_lbs(counts, capacity=None):
    c = torch.as_tensor(np.asarray(counts, np.int32), device="cuda")
    total = int(np.sum(np.asarray(counts, np.int64)))
    cap = total if capacity is None else capacity
    scanned = torch.empty(max(len(counts), 1), dtype=torch.int32, device="cuda")
    result = torch.empty(max(cap, 0), dtype=torch.int32, device="cuda")
    tdev = torch.full((1,), -1, dtype=torch.int32, device="cuda")
    t = gu.lbs(c, scanned, result, total_dev=tdev)
    torch.cuda.synchronize()
    return scanned[: len(counts)].cpu().numpy(), result[:t].cpu().numpy(), t, int(tdev.item())


@pytest.mark.parametrize("name", golden_names("lbs_"))
def test_lbs_golden(name):
    g = load_golden(name, "lbs_")
    scanned, result, total, tdev = run_lbs(g["counts"])
    assert total == tdev == int(g["counts"].sum())
    np.testing.assert_array_equal(scanned, g["scanned"])
    np.testing.assert_array_equal(result, g["result"])


# 6,000,017 counts are 733 scan tiles: more CTAs than the GPU holds at once, so the
# dependent launches start only after the scan's last CTAs have begun
@pytest.mark.parametrize("seed,N,hi", [(1, 1_000_003, 8), (2, 50_000, 2000), (3, 4097, 1), (4, 123_457, 0),
                                       (5, 6_000_017, 3)])
def test_lbs_random_vs_oracle(seed, N, hi):
    rng = np.random.default_rng(seed)
    counts = rng.integers(0, hi + 1, N).astype(np.int32)
    counts[rng.random(N) < 0.3] = 0
    scanned, result, total, _ = run_lbs(counts)
    rs, rr, rt = oracle.lbs(counts)
    assert total == rt
    np.testing.assert_array_equal(scanned, rs)
    np.testing.assert_array_equal(result, rr)


@pytest.mark.parametrize("c_off,s_off,r_off", [(1, 0, 0), (0, 3, 1), (3, 1, 2), (2, 2, 3)])
def test_lbs_unaligned_views(c_off, s_off, r_off):
    """Counts, scanned and result as views at element offsets from their buffers'
    16-byte-aligned starts: the owners' 16-byte stores realign to the result
    buffer, and nothing outside the views is written."""
    rng = np.random.default_rng(10 + c_off + 4 * r_off)
    N = 70_001
    counts = rng.integers(0, 6, N).astype(np.int32)
    total = int(counts.sum())
    cbuf = torch.zeros(N + 8, dtype=torch.int32, device="cuda")
    cbuf[c_off:c_off + N] = torch.as_tensor(counts, device="cuda")
    sbuf = torch.full((N + 8,), -5, dtype=torch.int32, device="cuda")
    rbuf = torch.full((total + 8,), -5, dtype=torch.int32, device="cuda")
    t = gu.lbs(cbuf[c_off:c_off + N], sbuf[s_off:s_off + N], rbuf[r_off:r_off + total])
    rs, rr, rt = oracle.lbs(counts)
    assert t == rt == total
    np.testing.assert_array_equal(sbuf[s_off:s_off + N].cpu().numpy(), rs)
    np.testing.assert_array_equal(rbuf[r_off:r_off + total].cpu().numpy(), rr)
    assert bool((sbuf[:s_off] == -5).all()) and bool((sbuf[s_off + N:] == -5).all())
    assert bool((rbuf[:r_off] == -5).all()) and bool((rbuf[r_off + total:] == -5).all())


def test_lbs_grid_degree_array():
    hg = gu.HostGraph.grid(2048, 2048, 0.05, seed=7)
    counts = np.diff(hg.R).astype(np.int32)
    scanned, result, total, _ = run_lbs(counts)
    assert 0.0 < gu.lbs_last_ms() < 100.0  # the call's device time (events around its kernels)
    rs, rr, rt = oracle.lbs(counts)
    assert total == rt == hg.m
    np.testing.assert_array_equal(scanned, rs)
    np.testing.assert_array_equal(result, rr)


def test_lbs_errors():
    L = gu.lib()
    with pytest.raises(gu.GuError) as e:
        run_lbs(np.full(4, 2 ** 30, np.int32), capacity=16)
    assert e.value.status == 5  # overflow
    with pytest.raises(gu.GuError) as e:
        run_lbs(np.full(10, 5, np.int32), capacity=20)
    assert e.value.status == 4 and b"50" in L.gu_last_error()
    with pytest.raises(gu.GuError) as e:
        run_lbs(np.array([3, -1, 4], np.int32), capacity=6)
    assert e.value.status == 1
    # a rejected call leaves the result slots and the device total as they were
    for counts, cap in ((np.full(10, 5, np.int32), 20), (np.array([3, -1, 4], np.int32), 6)):
        c = torch.as_tensor(counts, device="cuda")
        sc = torch.empty_like(c)
        res = torch.full((cap,), -7, dtype=torch.int32, device="cuda")
        tot = torch.full((1,), -9, dtype=torch.int32, device="cuda")
        with pytest.raises(gu.GuError):
            gu.lbs(c, sc, res, total_dev=tot)
        assert bool((res == -7).all()) and int(tot.item()) == -9
    # no items
    c = torch.zeros(0, dtype=torch.int32, device="cuda")
    assert gu.lbs(c, torch.zeros(1, dtype=torch.int32, device="cuda"), torch.zeros(0, dtype=torch.int32,
                                                                                      device="cuda")) == 0


def test_lbs_total_at_int32_max():
    """The largest total the int32 offsets hold: 4096 items owning 2^31 - 1 slots
    (an 8 GiB result).  Checked through size-independent properties: the scan is
    exact, owners never decrease, each item owns exactly its count of slots and
    its first slot sits at its offset.  One slot more overflows."""
    N, per = 4096, 1 << 19
    counts = np.full(N, per, np.int32)
    c = torch.as_tensor(counts, device="cuda")
    sc = torch.empty_like(c)
    small = torch.full((16,), -7, dtype=torch.int32, device="cuda")
    with pytest.raises(gu.GuError) as e:
        gu.lbs(c, sc, small)  # total 2^31
    assert e.value.status == 5 and bool((small == -7).all())
    counts[-1] -= 1
    c = torch.as_tensor(counts, device="cuda")
    total = (1 << 31) - 1
    res = torch.empty(total, dtype=torch.int32, device="cuda")
    tdev = torch.zeros(1, dtype=torch.int32, device="cuda")
    assert gu.lbs(c, sc, res, total_dev=tdev) == total
    assert int(tdev.item()) == total
    offs = torch.arange(N, device="cuda", dtype=torch.int64) * per
    assert torch.equal(sc.to(torch.int64), offs)
    assert torch.equal(res[offs].to(torch.int64), torch.arange(N, device="cuda", dtype=torch.int64))
    owned = torch.zeros(N, dtype=torch.int64, device="cuda")
    chunk = 1 << 28
    for s0 in range(0, total, chunk):
        part = res[s0:min(total, s0 + chunk + 1)]  # one slot of overlap for the order check
        assert bool((part[1:] >= part[:-1]).all())
        owned += torch.bincount(res[s0:min(total, s0 + chunk)].to(torch.int64), minlength=N)
    assert torch.equal(owned, c.to(torch.int64))
    del res
    torch.cuda.empty_cache()


def test_race_and_resolve_vs_oracle():
    rng = np.random.default_rng(5)
    nw = 4096
    pred = (rng.random(nw * 32) < rng.choice([0.0, 0.03, 0.5, 1.0], nw).repeat(32)).astype(np.int32)
    p = torch.as_tensor(pred, device="cuda")
    w = torch.empty_like(p)
    gu.race_and_resolve(p, w)
    got = w.cpu().numpy()
    for g in range(nw):
        vote = 0
        for l in range(32):
            if pred[32 * g + l]:
                vote |= 1 << l
        for l in range(32):
            assert got[32 * g + l] == oracle.race_and_resolve(vote, l)
