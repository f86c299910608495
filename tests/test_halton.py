"""halton::sample(index, dimension) of sub_crates/halton (Halton points with
Faure permutations, generated by sub_crates/halton/build.rs).  The oracle's
C++ restatement is pinned against known answers (dimension 0 is the base-2
radical inverse; dimensions whose Faure permutation is the identity on the
digits used give the plain radical inverse) and against an independent
Python restatement of the generator on every dimension; the GPU library's
psy_halton_samples must equal the oracle bit for bit."""
import ctypes as C
from fractions import Fraction

import numpy as np
import pytest


def _primes(n):
    out, c = [], 1
    while len(out) < n:
        c += 1
        if all(c % q for q in range(2, int(c ** 0.5) + 1)):
            out.append(c)
    return out


def _faure(bmax):
    f = [[0], [0], [0, 1]]
    for b in range(3, bmax + 1):
        if b % 2:
            c = (b - 1) // 2
            p = []
            for i in range(b):
                if i == c:
                    p.append(c)
                else:
                    v = f[b - 1][i - (1 if i > c else 0)]
                    p.append(v + (1 if v >= c else 0))
        else:
            c = b // 2
            p = [2 * f[c][i] for i in range(c)] + [2 * f[c][i] + 1 for i in range(c)]
        f.append(p)
    return f


PRIMES = _primes(128)
FAURE = _faure(PRIMES[-1])


def py_sample(index, dim):
    """Independent Python restatement: exact integer digit sums, f32 ops by numpy."""
    if dim == 0:
        rev = int("{:032b}".format(index)[::-1], 2)
        return np.float32(rev) * np.float32(1.0 / 4294967296.0)
    b = PRIMES[dim]
    pb, digits = b, 1
    while pb * b <= 500:
        pb *= b
        digits += 1
    mp = pb
    while mp * pb < (1 << 32):
        mp *= pb

    def perm(j):
        r = 0
        for _ in range(digits):
            r = r * b + FAURE[b][j % b]
            j //= b
        return r
    groups, total, w, rest = 0, 0, mp // pb, index
    while w >= 1:
        total += perm(rest % pb) * w
        rest //= pb
        w //= pb
        groups += 1
    scale = np.float32(np.float32(0.999999940395355224609375) / np.float32(mp))
    return np.float32(np.float32(total) * scale)


def oracle_sample(lib, index, dim):
    v = C.c_float()
    assert lib.psyo_halton_sample(index, dim, C.byref(v)) == 0
    return np.float32(v.value)


def test_faure_permutations_known():
    # published Faure permutations of small bases
    assert FAURE[3] == [0, 1, 2]
    assert FAURE[4] == [0, 2, 1, 3]
    assert FAURE[5] == [0, 3, 2, 1, 4]
    assert FAURE[7] == [0, 2, 5, 3, 1, 4, 6]


def test_oracle_known_answers(oracle_lib):
    # dimension 0: van der Corput in base 2 (bit reversal, times 2^-32)
    for i, v in [(0, 0.0), (1, 0.5), (2, 0.25), (3, 0.75), (5, 0.625)]:
        assert oracle_sample(oracle_lib, i, 0) == np.float32(v)
    # dimension 1 (base 3, Faure permutation the identity): the radical
    # inverse, scaled by 0.99999994 in f32
    for i in [1, 2, 3, 4, 10, 242, 243, 1000]:
        num, den, j = 0, 1, i
        while j:
            den *= 3
            num = num * 3 + j % 3
            j //= 3
        exact = Fraction(num, den)
        mp = 243 ** 4
        total = exact * mp
        assert total.denominator == 1
        want = np.float32(np.float32(int(total)) * np.float32(np.float32(0.999999940395355224609375) / np.float32(mp)))
        assert oracle_sample(oracle_lib, i, 1) == want, i
    v = C.c_float()
    assert oracle_lib.psyo_halton_sample(0, 128, C.byref(v)) == -1


def test_oracle_matches_python_restatement(oracle_lib):
    rng = np.random.default_rng(5)
    idx = [0, 1, 2, 3, 7, 499, 500, 65535, 65536, 2 ** 31, 2 ** 32 - 1] + [int(x) for x in rng.integers(0, 2 ** 32, 20)]
    for dim in range(128):
        for i in idx:
            a, b = oracle_sample(oracle_lib, i, dim), py_sample(i, dim)
            assert a.tobytes() == b.tobytes(), (dim, i, a, b)
            # the generated code's f32 conversion of a sum near (b^d)^K can
            # round the product up to exactly 1.0 despite its "[0,1)" note
            assert 0.0 <= a <= 1.0


@pytest.mark.gpu
def test_gpu_halton_bit_exact(gpu_lib, oracle_lib):
    from psychopath_gb300 import gpu
    rng = np.random.default_rng(7)
    idx = np.concatenate([np.arange(0, 1024, dtype=np.uint32),
                          np.array([2 ** 32 - 1, 2 ** 31, 65535, 65536], dtype=np.uint32),
                          rng.integers(0, 2 ** 32, 1024, dtype=np.uint64).astype(np.uint32)])
    for dim in range(128):
        got = gpu.halton_samples(dim, idx)
        want = np.array([oracle_sample(oracle_lib, int(i), dim) for i in idx], dtype=np.float32)
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), dim
    with pytest.raises(gpu.PsyError):
        gpu.halton_samples(128, idx[:4])
