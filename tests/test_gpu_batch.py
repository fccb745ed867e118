"""GPU parity of the batched executor (af_batch_*) against the oracle.

The batch mixes every execution scheme: single-tile transforms (split-radix,
Good-Thomas, Rader with a smooth or a zero-padded convolution, Bluestein) and
multi-pass transforms (four-step, two-pass Good-Thomas, three-pass Rader and
Bluestein convolutions).  Each transform is compared with the oracle's
Planned.transform in FP64.
"""
import numpy as np
import pytest

from _util import crand, fp32_bound, rel_l2

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

# tiles: plain, GT, Rader (smooth p-1), Rader (padded), Bluestein;
# multi-pass: four-step SR / CT, GT two-pass, Rader conv (smooth / padded), Bluestein conv
SIZES = [1, 2, 3, 4, 5, 7, 8, 13, 16, 17, 47, 83, 100, 257, 307, 1001, 1009, 1031, 4096, 4099, 8192, 12289,
         16384, 19683, 20000, 15015, 13007, 65536, 65537, 30011, 26701, 49999]


def O():
    from oracle import oracle
    return oracle


def make_batch(sizes, sign=-1):
    from accelerate_fourier import _lib
    return _lib.Batch(sizes, sign)


def run(b, x, fn="exec"):
    xd = torch.from_numpy(x.astype(np.complex64)).cuda()
    y = torch.empty_like(xd)
    s = torch.cuda.current_stream().cuda_stream
    getattr(b, fn + "_ptr")(xd.data_ptr(), y.data_ptr(), s)
    torch.cuda.synchronize()
    return y.cpu().numpy()


def split(v, sizes):
    offs = np.concatenate([[0], np.cumsum(sizes)[:-1]])
    return [v[o:o + n] for o, n in zip(offs, sizes)]


def test_plan_kinds_present():
    kinds = {O().plan_string(n)[:2].rstrip("0123456789") for n in SIZES}
    assert {"SR", "GT", "P", "BL", "CT"} <= kinds


@pytest.mark.parametrize("sign", [-1, 1])
def test_batch_forward_matches_oracle(sign):
    sizes = np.array(SIZES, dtype=np.int64)
    rng = np.random.default_rng(11)
    x = crand(rng, int(sizes.sum()), "normal")
    b = make_batch(sizes, sign)
    y = run(b, x)
    for n, xi, yi in zip(sizes, split(x, sizes), split(y, sizes)):
        ref = O().planned(xi[None], sign)[0]
        assert rel_l2(yi, ref) <= fp32_bound(n, 4.0), (int(n), O().plan_string(int(n))[:40], rel_l2(yi, ref))


def test_batch_vjp_matches_oracle():
    sizes = np.array(SIZES, dtype=np.int64)
    rng = np.random.default_rng(12)
    g = crand(rng, int(sizes.sum()), "normal")
    b = make_batch(sizes, -1)
    y = run(b, g, "vjp")
    for n, gi, yi in zip(sizes, split(g, sizes), split(y, sizes)):
        ref = O().planned(gi[None], +1)[0]
        assert rel_l2(yi, ref) <= fp32_bound(n, 4.0), int(n)


def test_batch_forward_cotangent():
    sizes = np.array(SIZES, dtype=np.int64)
    rng = np.random.default_rng(13)
    total = int(sizes.sum())
    x = crand(rng, total, "normal")
    w = rng.uniform(0, 1, total)
    b = make_batch(sizes, -1)
    xd = torch.from_numpy(x.astype(np.complex64)).cuda()
    wd = torch.from_numpy(w.astype(np.float32)).cuda()
    cot = torch.empty_like(xd)
    loss = torch.zeros(1, dtype=torch.float64, device="cuda")
    b.forward_cotangent_ptr(xd.data_ptr(), wd.data_ptr(), cot.data_ptr(), loss.data_ptr(),
                            torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    c = cot.cpu().numpy()
    ref_loss = 0.0
    for n, xi, wi, ci in zip(sizes, split(x, sizes), split(w, sizes), split(c, sizes)):
        X = O().planned(xi[None], -1)[0]
        ref_loss += float(np.sum(wi * np.abs(X) ** 2))
        assert rel_l2(ci, 2 * wi * X) <= fp32_bound(n, 4.0), int(n)
    assert abs(loss.item() - ref_loss) <= 1e-5 * ref_loss


def test_batch_repeated_lengths_and_zero():
    sizes = np.array([0, 64, 64, 0, 1000, 64, 65537, 65537, 3], dtype=np.int64)
    rng = np.random.default_rng(14)
    x = crand(rng, int(sizes.sum()), "normal")
    y = run(make_batch(sizes, -1), x)
    for n, xi, yi in zip(sizes, split(x, sizes), split(y, sizes)):
        if n:
            assert rel_l2(yi, O().planned(xi[None], -1)[0]) <= fp32_bound(n, 4.0)


def test_benchmark_workload_sample():
    """The benchmark's 4096 mixed lengths: every 64th transform vs the oracle,
    and the launch count stays small."""
    import bench
    sizes = bench.workload_sizes()
    b = make_batch(sizes, -1)
    assert b.launches() == 1  # one persistent launch per call
    rng = np.random.default_rng(5)
    x = crand(rng, int(sizes.sum()), "normal")
    y = run(b, x)
    offs = np.concatenate([[0], np.cumsum(sizes)[:-1]])
    worst = 0.0
    for i in range(0, len(sizes), 64):
        n, o = int(sizes[i]), int(offs[i])
        ref = O().planned(x[o:o + n][None], -1)[0]
        err = rel_l2(y[o:o + n], ref)
        worst = max(worst, err)
        assert err <= fp32_bound(n, 4.0), (n, err)
    assert worst < 1e-6


def test_batch_in_place():
    sizes = np.array([64, 1000, 4099, 20000, 30011], dtype=np.int64)
    rng = np.random.default_rng(15)
    x = crand(rng, int(sizes.sum()), "normal")
    b = make_batch(sizes, -1)
    xd = torch.from_numpy(x.astype(np.complex64)).cuda()
    b.exec_ptr(xd.data_ptr(), xd.data_ptr(), torch.cuda.current_stream().cuda_stream)
    b.status(torch.cuda.current_stream().cuda_stream)
    y = xd.cpu().numpy()
    for n, xi, yi in zip(sizes, split(x, sizes), split(y, sizes)):
        assert rel_l2(yi, O().planned(xi[None], -1)[0]) <= fp32_bound(n, 4.0), int(n)


def test_lengths_beyond_the_executor_use_the_multi_launch_plan():
    """A Bluestein length above 131072 runs on the multi-launch batch plan."""
    sizes = np.array([200003, 64], dtype=np.int64)
    rng = np.random.default_rng(16)
    x = crand(rng, int(sizes.sum()), "normal")
    b = make_batch(sizes, -1)
    assert b.launches() > 1
    y = run(b, x)
    for n, xi, yi in zip(sizes, split(x, sizes), split(y, sizes)):
        assert rel_l2(yi, O().planned(xi[None], -1)[0]) <= fp32_bound(n, 4.0), int(n)


def test_stage_wait_timeout_is_reported_and_the_device_stays_usable():
    """A work item whose previous stage never reaches its count gives up after
    a bounded number of polls: the launch ends, af_batch_status reports
    AF_ERR_TIMEOUT, and the next batch runs normally."""
    import ctypes
    from accelerate_fourier import _lib
    sizes = np.array([30011, 20000, 64], dtype=np.int64)
    b = make_batch(sizes, -1)
    L = _lib.load()
    L.afx_batch_poison_wait.argtypes = [ctypes.c_void_p, ctypes.c_longlong]
    assert L.afx_batch_poison_wait(b._h, 20000) == 0
    x = torch.ones(int(sizes.sum()), dtype=torch.complex64, device="cuda")
    y = torch.empty_like(x)
    s = torch.cuda.current_stream().cuda_stream
    b.exec_ptr(x.data_ptr(), y.data_ptr(), s)
    with pytest.raises(_lib.AfError) as e:
        b.status(s)
    assert e.value.code == 5  # AF_ERR_TIMEOUT
    rng = np.random.default_rng(17)
    xs = crand(rng, int(sizes.sum()), "normal")
    ys = run(make_batch(sizes, -1), xs)
    for n, xi, yi in zip(sizes, split(xs, sizes), split(ys, sizes)):
        assert rel_l2(yi, O().planned(xi[None], -1)[0]) <= fp32_bound(n, 4.0), int(n)


def test_tuned_batch_matches_oracle_and_reuses_its_cache(tmp_path):
    """af_batch_create_tuned times candidate planner choices on the device,
    keeps the winner in the cache file, and a second creation reuses it."""
    from accelerate_fourier import _lib
    sizes = np.array([64, 1000, 4099, 20000, 30011, 16000, 65536], dtype=np.int64)
    cache = tmp_path / "tune.jsonl"
    b = _lib.Batch(sizes, -1, tune_cache=cache)
    d = b.describe()
    assert d["executor"] == "persistent"
    assert d["autotune"]["ms"] <= d["autotune"]["default_ms"]
    assert d["tuning"] == d["autotune"]["tune"]
    assert cache.exists() and len(cache.read_text().splitlines()) == 1
    b2 = _lib.Batch(sizes, -1, tune_cache=cache)
    assert b2.describe()["autotune"] == "cached"
    assert b2.describe()["tuning"] == d["tuning"]
    rng = np.random.default_rng(18)
    x = crand(rng, int(sizes.sum()), "normal")
    y = run(b2, x)
    for n, xi, yi in zip(sizes, split(x, sizes), split(y, sizes)):
        assert rel_l2(yi, O().planned(xi[None], -1)[0]) <= fp32_bound(n, 4.0), int(n)
