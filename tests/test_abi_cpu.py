"""CPU checks of the native layer: the library loads and exports every entry
point of include/atm.h, and the kernels' FFT / Bessel / phase arithmetic (run
on the host through libatm_selftest.so) is right."""
import ctypes
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def built():
    from pyatmosphere_gb300 import build
    return build.build()


def declared_symbols():
    src = open(os.path.join(ROOT, "include", "atm.h")).read()
    return sorted(set(re.findall(r"^\s*(?:int|int64_t|const char\*)\s+(atm_\w+)\s*\(", src, re.M)))


def test_library_exports_every_declared_symbol(built):
    lib = ctypes.CDLL(built["libatm"])
    names = declared_symbols()
    assert len(names) >= 8
    for n in names:
        assert hasattr(lib, n), n
    from pyatmosphere_gb300.engine import _lib
    assert set(names) == set(_lib.SIGNATURES), "ctypes signatures must cover include/atm.h"
    lib.atm_abi_version.restype = ctypes.c_int
    assert lib.atm_abi_version() == _lib.ABI_VERSION == 3


def test_plan_create_rejects_bad_descriptors_without_gpu(built):
    from pyatmosphere_gb300.engine import _lib
    lib = _lib.load(built["libatm"])
    d = _lib.AtmChannelDesc()
    d.abi_version = _lib.ABI_VERSION
    d.resolution = 100          # not a power of two
    d.delta, d.wvl, d.w0, d.batch = 1e-3, 8e-7, 0.1, 1
    h = ctypes.c_void_p()
    assert lib.atm_plan_create(ctypes.byref(d), ctypes.byref(h)) == -2
    assert b"resolution" in lib.atm_last_error()
    d.resolution, d.abi_version = 256, 7
    assert lib.atm_plan_create(ctypes.byref(d), ctypes.byref(h)) == -1
    assert lib.atm_autotune(None, 1, 1, None) == -1
    assert lib.atm_plan_set_variants(None, 0, 4, 0) == -1
    assert b"NULL" in lib.atm_last_error()


@pytest.mark.parametrize("N", [64, 128, 256, 512, 1024, 2048, 4096])
def test_kernel_fft_arithmetic_on_host(built, N):
    from pyatmosphere_gb300.engine._lib import load_selftest
    lib = load_selftest(built["selftest"])
    rng = np.random.default_rng(N)
    x = (rng.standard_normal(N) + 1j * rng.standard_normal(N)).astype(np.complex64)
    for d in (-1, 1):
        ref = np.fft.fft(x.astype(np.complex128)) if d < 0 else np.fft.ifft(x.astype(np.complex128)) * N
        out = np.zeros(N, np.complex64)
        assert lib.atm_selftest_fft(N, d, x.ctypes.data, out.ctypes.data) == 0
        assert np.linalg.norm(out - ref) / np.linalg.norm(ref) < 3e-7
        # twiddles formed from powers of two (column-pass variant 2): a few ulp more
        out2 = np.zeros(N, np.complex64)
        assert lib.atm_selftest_fft_twrec(N, d, x.ctypes.data, out2.ctypes.data) == 0
        assert np.linalg.norm(out2 - ref) / np.linalg.norm(ref) < 5e-7
        # twiddle bases held per thread (the register-twiddle passes): the same bits
        out3 = np.zeros(N, np.complex64)
        assert lib.atm_selftest_fft_twreg(N, d, x.ctypes.data, out3.ctypes.data) == 0
        np.testing.assert_array_equal(out3, out2)


@pytest.mark.parametrize("N", [1024, 2048, 4096])
def test_warp_fft_arithmetic_on_host(built, N):
    """The warp FFT of the row / column pass forms 11 / 10 (one exchange per
    transform, lanes emulated on the host; 64 lanes at 4096) against numpy in
    FP64; every exchange swizzle gives the same bits."""
    from pyatmosphere_gb300.engine._lib import load_selftest
    lib = load_selftest(built["selftest"])
    rng = np.random.default_rng(N + 1)
    x = (rng.standard_normal(N) + 1j * rng.standard_normal(N)).astype(np.complex64)
    for d in (-1, 1):
        ref = np.fft.fft(x.astype(np.complex128)) if d < 0 else np.fft.ifft(x.astype(np.complex128)) * N
        outs = []
        for mode in ((1, 2) if N == 4096 else range(5)):
            out = np.zeros(N, np.complex64)
            assert lib.atm_selftest_wfft(N, d, mode, x.ctypes.data, out.ctypes.data) == 0
            outs.append(out)
        assert np.linalg.norm(outs[0] - ref) / np.linalg.norm(ref) < 3e-7
        for out in outs[1:]:
            np.testing.assert_array_equal(out, outs[0])
    assert lib.atm_selftest_wfft(512, -1, 0, x.ctypes.data, x.ctypes.data) == -1


def _wfft_slot(kb, jj, sw):
    return kb * 32 + (jj ^ sw)


@pytest.mark.parametrize("R", [32, 64])
def test_warp_fft_exchange_is_bank_conflict_free(R):
    """Each half warp's eight-byte stores and loads of the warp-FFT exchange
    land on 16 distinct bank pairs, for the row pass (a warp = one transform's
    32 lanes) and the column pass (a warp = 8 lanes of each of 4 columns);
    the slots of a transform are a permutation of its N slots."""
    N = 32 * R
    half_warps = [range(0, 16), range(16, 32)]
    # row pass: lane j of the warp is the transform's lane j
    for kb in range(R):
        for hw in half_warps:
            assert len({_wfft_slot(kb, j, kb & 15) % 16 for j in hw}) == 16
    for h in range(R // 32):
        for jj in range(32):
            for hw in half_warps:
                assert len({_wfft_slot(j + 32 * h, jj, (j + 32 * h) & 15) % 16 for j in hw}) == 16
    assert sorted(_wfft_slot(kb, jj, kb & 15) for kb in range(R) for jj in range(32)) == list(range(N))
    # column pass: lane (a = lane // 4, c = lane % 4) of warp w is lane j = 8 w + a of column c,
    # whose exchange rows start at slot c N
    for w in range(4):
        for kb in range(R):
            for hw in half_warps:
                slots = {(c * N + _wfft_slot(kb, 8 * w + lane // 4, (kb & 3) | (c << 2))) % 16
                         for lane in hw for c in [lane % 4]}
                assert len(slots) == 16
        for h in range(R // 32):
            for jj in range(32):
                for hw in half_warps:
                    slots = set()
                    for lane in hw:
                        c, kb = lane % 4, 8 * w + lane // 4 + 32 * h
                        slots.add((c * N + _wfft_slot(kb, jj, (kb & 3) | (c << 2))) % 16)
                    assert len(slots) == 16
    for c in range(4):
        assert sorted(_wfft_slot(kb, jj, (kb & 3) | (c << 2)) for kb in range(R) for jj in range(32)) == list(range(N))
    # the tile read / write-back: instruction m of warp w covers 32 consecutive slots
    for w in range(4):
        for m in range(R):
            slots = [(32 * m + 8 * w + lane // 4) * 4 + lane % 4 for lane in range(32)]
            assert slots == list(range(slots[0], slots[0] + 32))


def test_warp_fft_4096_exchange_is_bank_conflict_free():
    """N = 4096 (64-lane transforms, R = 64): lane (a = lane // 2, c = lane % 2)
    of warp w is lane j = 16 w + a of column c of a two-column tile; its
    exchange (swizzle (kb & 7) | (c << 3)) and the tile read are free of bank
    conflicts per half warp, and the slots of a column are a permutation."""
    L, R, N = 64, 64, 4096
    half_warps = [range(0, 16), range(16, 32)]

    def slot(kb, jj, c):
        return c * N + kb * L + (jj ^ ((kb & 7) | (c << 3)))

    for w in range(4):
        for kb in range(R):
            for hw in half_warps:
                assert len({slot(kb, 16 * w + lane // 2, lane % 2) % 16 for lane in hw}) == 16
        for jj in range(L):
            for hw in half_warps:
                assert len({slot(16 * w + lane // 2, jj, lane % 2) % 16 for lane in hw}) == 16
        for m in range(R):
            slots = [(L * m + 16 * w + lane // 2) * 2 + lane % 2 for lane in range(32)]
            assert slots == list(range(slots[0], slots[0] + 32))
    for c in range(2):
        assert sorted(slot(kb, jj, c) - c * N for kb in range(R) for jj in range(L)) == list(range(N))


def test_bessel_coefficients_on_host(built):
    from scipy.special import jv
    from pyatmosphere_gb300.engine._lib import load_selftest
    lib = load_selftest(built["selftest"])
    J = np.zeros(64)
    for a in [1e-9, 1e-3, 0.7, 3.1, -9.4, 25.0]:
        assert lib.atm_selftest_bessel(a, 64, J.ctypes.data) == 0
        np.testing.assert_allclose(J, jv(np.arange(64), a), atol=1e-14)


def test_fixed_point_phase_wrap_on_host(built):
    """frac(j S + O) through 64-bit fixed point agrees with exact rational
    arithmetic to float32 resolution, including phases of ~1e3 turns."""
    from pyatmosphere_gb300.engine._lib import load_selftest
    lib = load_selftest(built["selftest"])
    from fractions import Fraction
    for S, O in [(0.4999321, -512.25), (1e-7, 3.3), (0.123456789, -0.7)]:
        out = np.zeros(4096, np.float32)
        lib.atm_selftest_turns(S, O, 4096, out.ctypes.data)
        for j in [0, 1, 17, 2047, 4095]:
            t = Fraction(S) * j + Fraction(O)
            frac = float(t - (t.numerator // t.denominator))
            ref = frac if frac < 0.5 else frac - 1.0
            got = out[j] / 2.0
            assert abs(((got - ref) + 0.5) % 1.0 - 0.5) < 2e-7
