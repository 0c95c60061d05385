"""CPU-only checks: oracle pins, generators, math primitives, the library's
exported symbols and the file surface.  No GPU call is made here."""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

from tests import cases

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_library_exports_every_header_symbol(mcfl_lib):
    hdr = open(os.path.join(ROOT, "include", "mcfl.h")).read()
    declared = sorted(set(re.findall(r"\b(mcfl_[A-Za-z_0-9]+)\s*\(", hdr)))
    assert len(declared) > 20
    for name in declared:
        assert hasattr(mcfl_lib, name), name


def test_safeprime_generators_agree(mcfl_lib, oracle, multipliers, tmp_path):
    p = tmp_path / "sp.txt"
    assert mcfl_lib.mcfl_write_safeprimes(str(p).encode(), 32769) == 0
    prod = np.loadtxt(p, dtype=np.uint64)
    assert prod.shape == (32769, 3)
    assert np.array_equal(prod[:, 0].astype(np.uint32), multipliers)
    assert multipliers[0] == 4294967118  # largest a < 2^32 with a*2^32-1, a*2^31-1 prime
    assert np.all(np.diff(multipliers.astype(np.int64)) < 0)


def _is_prime(n):
    if n < 2:
        return False
    d, s = n - 1, 0
    while d % 2 == 0:
        d //= 2
        s += 1
    for a in (2, 3, 5, 7, 11, 13, 17, 19, 23, 29, 31, 37):
        x = pow(a, d, n)
        if x in (1, n - 1):
            continue
        for _ in range(s - 1):
            x = x * x % n
            if x == n - 1:
                break
        else:
            return False
    return True


def test_safeprime_criterion_spot_check(multipliers):
    for a in list(multipliers[:5]) + list(multipliers[-3:]):
        a = int(a)
        assert _is_prime(a * 2**32 - 1) and _is_prime(a * 2**31 - 1)
    # nothing valid was skipped above the first entry
    for a in range(int(multipliers[0]) + 1, 2**32):
        assert not (_is_prime(a * 2**31 - 1) and _is_prime(a * 2**32 - 1))


def test_portable_math_accuracy(oracle):
    L = oracle.lib
    L.oracle_plogf.restype = ctypes.c_float
    L.oracle_plogf.argtypes = [ctypes.c_float]
    L.oracle_psincosf.argtypes = [ctypes.c_float, ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_float)]
    rng = np.random.default_rng(0)
    u = np.concatenate([rng.random(20000), [2.0**-24, 0.5, 1.0 - 2**-24, 1.0]]).astype(np.float32)
    worst = 0.0
    for v in u:
        got = L.oracle_plogf(float(v))
        exact = np.log(np.float64(v))
        if exact != 0:
            ulp = np.spacing(np.float32(abs(exact)))
            worst = max(worst, abs(got - exact) / ulp)
        else:
            assert got == 0.0
    assert worst < 3.0
    s, c = ctypes.c_float(), ctypes.c_float()
    for v in (rng.random(20000) * 2 * np.pi).astype(np.float32):
        L.oracle_psincosf(float(v), ctypes.byref(s), ctypes.byref(c))
        assert abs(s.value - np.sin(np.float64(v))) < 2.5e-7
        assert abs(c.value - np.cos(np.float64(v))) < 2.5e-7


def test_line_sphere_known_answer(oracle):
    """FoundBoundaryPython.ipynb:33,38: p=(0.8,1.2,1), d=(0,0,1), c=(1,1,1),
    r=0.5 gives the distances -+0.412310562562 (= sqrt(0.17))."""
    L = oracle.lib
    f3 = ctypes.c_float * 3
    out = (ctypes.c_float * 2)()
    L.oracle_sphere_back_steps(f3(0.8, 1.2, 1.0), f3(0.0, 0.0, 1.0), f3(1.0, 1.0, 1.0), ctypes.c_float(0.25), out)
    assert sorted([out[0], out[1]]) == pytest.approx([-0.412310562562, 0.412310562562], abs=2e-7)


def test_oracle_photon_mode_conserves_weight_exactly(oracle, table32768):
    case = cases.mismatch(photons=20000, per_voxel=200)
    r = oracle.run_photon(case.oracle_sim(), table32768, 3, 4, libm=False)
    a, top, bottom, rl, rg, w0 = r.balance
    assert (a + top + bottom + rl + w0 - rg) % 2**64 == r.photons_exc * case.start_weight()
    assert r.Rd.sum() <= top and r.Tt.sum() <= bottom
