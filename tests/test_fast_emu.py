"""The batched executor's work items run on the CPU.

libaf compiles the persistent executor's item code for the host as well; the
host emulator runs every work item of a batch in queue order, one thread index
at a time per phase, with exactly the shared memory the item's shape reserves.
These tests check, without a GPU, that the planner's items (direct, Bluestein,
four-step and three-pass Bluestein stages) compute the transform the oracle
computes (Planned.transform in FP64), for every tuning the autotuner may pick,
and that a wait on a stage that never completes reports a timeout.
"""
import ctypes
import os

import numpy as np
import pytest

from _util import crand, fp32_bound, rel_l2

P = ctypes.c_void_p


def lib():
    from accelerate_fourier import _build
    path = _build.LIB
    if not os.path.exists(path):
        pytest.skip("libaf.so is not built")
    L = ctypes.CDLL(path)
    L.afx_fast_create_tuned.argtypes = [P, ctypes.c_int64, ctypes.c_int, P, ctypes.c_int, ctypes.POINTER(P)]
    L.afx_fast_exec.argtypes = [P, ctypes.c_int, P, P, P, P, P]
    L.afx_fast_error.restype = ctypes.c_char_p
    L.afx_fast_status.argtypes = [P, P]
    L.afx_fast_destroy.argtypes = [P]
    L.afx_fast_poison_wait.argtypes = [P, ctypes.c_longlong]
    L.afx_fast_describe.argtypes = [P, ctypes.c_char_p, ctypes.c_size_t]
    return L


def O():
    from oracle import oracle
    return oracle


class Emu:
    def __init__(self, sizes, tune=()):
        self.L = lib()
        self.sizes = np.ascontiguousarray(np.asarray(sizes, dtype=np.int64))
        t = np.ascontiguousarray(np.asarray(tune, dtype=np.int32))
        self.h = P()
        rc = self.L.afx_fast_create_tuned(self.sizes.ctypes.data, len(self.sizes), 1, t.ctypes.data if len(t) else None,
                                          len(t), ctypes.byref(self.h))
        assert rc == 0, self.L.afx_fast_error()

    def run(self, x, sign, w=None):
        x = np.ascontiguousarray(x.astype(np.complex64))
        y = np.zeros_like(x)
        loss = np.zeros(1)
        wp = np.ascontiguousarray(w.astype(np.float32)) if w is not None else None
        rc = self.L.afx_fast_exec(self.h, sign, x.ctypes.data, y.ctypes.data, wp.ctypes.data if wp is not None else None,
                                  loss.ctypes.data if wp is not None else None, None)
        assert rc == 0, self.L.afx_fast_error()
        return y, loss[0]

    def status(self):
        return self.L.afx_fast_status(self.h, None)

    def describe(self):
        import json
        buf = ctypes.create_string_buffer(4096)
        assert self.L.afx_fast_describe(self.h, buf, len(buf)) == 0
        return json.loads(buf.value.decode())

    def __del__(self):
        if getattr(self, "h", None):
            self.L.afx_fast_destroy(self.h)


def split(v, sizes):
    offs = np.concatenate([[0], np.cumsum(sizes)[:-1]])
    return [v[o:o + n] for o, n in zip(offs, sizes)]


# direct items (one and several transforms per CTA), Bluestein in one CTA,
# four-step (5-smooth beyond one CTA) and three-pass Bluestein (long primes)
SIZES = [0, 1, 2, 3, 5, 7, 8, 16, 16, 16, 27, 100, 100, 257, 1000, 1009, 4096, 6000, 7776, 12289, 16000,
         20000, 30011, 65536]
KINDS = ["direct", "blue", "cols", "rows", "bcols", "brows", "bcols2"]


def test_every_item_kind_planned():
    d = Emu(SIZES).describe()
    assert all(c > 0 for c in d["by_kind"]), dict(zip(KINDS, d["by_kind"]))


@pytest.mark.parametrize("sign", [-1, 1])
def test_emulated_batch_matches_oracle(sign):
    rng = np.random.default_rng(21)
    x = crand(rng, int(np.sum(SIZES)), "normal")
    y, _ = Emu(SIZES).run(x, sign)
    for n, xi, yi in zip(SIZES, split(x, SIZES), split(y, SIZES)):
        if n == 0:
            continue
        ref = O().planned(xi[None], sign)[0] if n <= 20000 else (np.fft.fft(xi) if sign < 0 else np.fft.ifft(xi) * n)
        assert rel_l2(yi, ref) <= fp32_bound(n, 4.0), (n, rel_l2(yi, ref))


def test_emulated_cotangent_epilogue():
    rng = np.random.default_rng(22)
    total = int(np.sum(SIZES))
    x = crand(rng, total, "normal")
    w = rng.uniform(0, 1, total)
    c, loss = Emu(SIZES).run(x, -1, w)
    ref_loss = 0.0
    for n, xi, wi, ci in zip(SIZES, split(x, SIZES), split(w, SIZES), split(c, SIZES)):
        if n == 0:
            continue
        X = np.fft.fft(xi)
        ref_loss += float(np.sum(wi * np.abs(X) ** 2))
        assert rel_l2(ci, 2 * wi * X) <= fp32_bound(n, 4.0), n
    assert abs(loss - ref_loss) <= 1e-5 * ref_loss


# (radix16, lines per multi-pass item, balanced lines per unit, item target, slack, L2 MB)
TUNES = [(0, 16, 1, 4096, 456, 48), (1, 32, 0, 4096, 912, 48), (1, 64, 1, 2048, 100, 8), (0, 8, 0, 8192, 5000, 512)]


@pytest.mark.parametrize("tune", TUNES)
def test_every_tuning_computes_the_same_transform(tune):
    sizes = [16, 100, 1000, 4096, 6000, 12289, 20000, 30011]
    rng = np.random.default_rng(23)
    x = crand(rng, int(np.sum(sizes)), "normal")
    y, _ = Emu(sizes, tune).run(x, -1)
    for n, xi, yi in zip(sizes, split(x, sizes), split(y, sizes)):
        assert rel_l2(yi, np.fft.fft(xi)) <= fp32_bound(n, 4.0), (tune, n)


def test_bad_tuning_is_rejected():
    L = lib()
    sizes = np.array([64], dtype=np.int64)
    t = np.array([1, 12, 0, 4096], dtype=np.int32)  # 12 lines: not a power of two
    h = P()
    assert L.afx_fast_create_tuned(sizes.ctypes.data, 1, 1, t.ctypes.data, len(t), ctypes.byref(h)) == 1
    assert b"power of two" in L.afx_fast_error()


def test_wait_that_never_completes_times_out():
    e = Emu([30011, 64])
    assert e.L.afx_fast_poison_wait(e.h, 1000) == 0
    e.run(np.ones(30011 + 64, dtype=np.complex64), -1)
    assert e.status() == 1  # FE_TIMEOUT


def test_no_wait_to_poison_in_single_stage_batches():
    e = Emu([64, 100])
    assert e.L.afx_fast_poison_wait(e.h, 1000) == 1
    e.run(np.ones(164, dtype=np.complex64), -1)
    assert e.status() == 0


def test_odd_lines_take_even_tiles():
    # 6561 = 81 x 81 and 50625 = 225 x 225 run four-step over odd line
    # lengths; with 3072-element items of up to 64 lines the planner would take 37 and 13
    # lines, tiles of an odd number of elements that cannot move as one bulk
    # copy: it takes an even count instead
    sizes = [6561, 50625]
    rng = np.random.default_rng(23)
    x = crand(rng, int(np.sum(sizes)), "normal")
    t = np.array([1, 64, 0, 3072, 2736, 48], dtype=np.int32)
    e = Emu(sizes, tune=t)
    assert e.describe()["by_kind"][2] > 0
    y, _ = e.run(x, -1)
    for n, xi, yi in zip(sizes, split(x, sizes), split(y, sizes)):
        assert rel_l2(yi, np.fft.fft(xi)) <= fp32_bound(n, 4.0), n
