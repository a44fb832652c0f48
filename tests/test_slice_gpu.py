"""Bit-exact parity of the split form's digit slicing (its integer work) against a
numpy restatement of the digit format, through orth_gb300_split_slice_dev:

  * each column's scale exponent e (max |x| < 2^e; Inf/NaN ignored; 0 for a zero
    column);
  * the fixed point V = round(x * 2^(8 planes - 1 - e)), half away from zero, from
    the FP64 bit pattern (zero for subnormals, Inf and NaN);
  * balanced base-256 digits d_0 (most significant) .. d_{planes-1}, stored as BF16
    bits;
  * the store's layout [plane][64-row chunk][column][64 rows], rows past m as
    digits of zero.

The cases cover both load paths of the slicing kernel (16-byte row pairs when
every column starts on a 16-byte boundary, single loads otherwise), partial row
tiles and chunks, a partial 16-column group, 6 and 7 planes, and ties, zeros,
subnormals, Inf and NaN.
"""
import numpy as np
import pytest

from bcgs_gb300 import orth

pytestmark = pytest.mark.gpu


def digits_reference(X: np.ndarray, planes: int):
    """Digit planes (planes, ceil(m/64), n, 64) as uint16 BF16 bits, and e per column."""
    m, n = X.shape
    bits = np.ascontiguousarray(X).view(np.int64)
    E = (bits >> 52) & 0x7FF
    absb = bits & 0x7FFFFFFFFFFFFFFF
    cmax = np.where(E == 0x7FF, 0, absb).max(axis=0)
    Ec = (cmax >> 52) & 0x7FF
    e = np.where(Ec == 0, 0, Ec - 1022)
    M = (bits & ((1 << 52) - 1)) | (1 << 52)
    sh = np.minimum(E - 1075 + 8 * planes - 1 - e[None, :], 9)
    up = M << np.clip(sh, 0, 9)
    rs = np.clip(-sh, 1, 62)
    down = (M + (np.int64(1) << (rs - 1))) >> rs
    V = np.where(sh >= 0, up, np.where(sh > -60, down, 0))
    V = np.where((E == 0) | (E == 0x7FF), 0, V)
    V = np.where(bits < 0, -V, V)
    bias = int(0x8080808080808080 >> (8 * (8 - (planes - 1))))
    Vb = V + bias
    d = np.empty((planes, m, n), dtype=np.int64)
    d[0] = Vb >> (8 * (planes - 1))
    for i in range(1, planes):
        d[i] = ((Vb >> (8 * (planes - 1 - i))) & 255) - 128
    bf = (d.astype(np.float32).view(np.uint32) >> 16).astype(np.uint16)
    nrc = (m + 63) // 64
    out = np.zeros((planes, nrc * 64, n), dtype=np.uint16)
    out[:, :m, :] = bf
    out = out.reshape(planes, nrc, 64, n).transpose(0, 1, 3, 2)
    return np.ascontiguousarray(out), e.astype(np.int32), V


def special_matrix(m: int, n: int, seed: int) -> np.ndarray:
    rng = np.random.default_rng(seed)
    X = rng.standard_normal((m, n)) * np.exp2(rng.integers(-40, 40, n))[None, :]
    X[rng.random((m, n)) < 0.02] = 0.0
    X[:, 1] = 0.0                                                   # a zero column
    X[:, 2] = 1.0                                                   # max exactly a power of two
    X[: m // 2, 2] = -0.75
    X[:, 3] = np.exp2(-1070.0) * rng.integers(1, 9, m)              # subnormals only
    X[5, 4] = np.inf                                                # Inf and NaN do not set the scale
    X[7, 4] = -np.inf
    X[9, 4] = np.nan
    # Ties: with column max 1.0 (e = 1) and 7 planes, x * 2^54 = k + 1/2.
    if n > 5:
        k = rng.integers(-(1 << 20), 1 << 20, m)
        X[:, 5] = (2.0 * k + 1.0) * np.exp2(-55.0)
        X[0, 5] = 1.0
    if n > 6:
        X[:, 6] = rng.standard_normal(m) * np.exp2(-60.0)          # tiny against the max
        X[0, 6] = 1e10
    return X


def run_slice(torch, X: np.ndarray, planes: int, ld: int):
    m, n = X.shape
    buf = torch.zeros((n, ld), dtype=torch.float64, device="cuda")
    buf[:, :m] = torch.from_numpy(np.ascontiguousarray(X.T))
    nrc = (m + 63) // 64
    dig = torch.full((planes * nrc * n * 64,), -1, dtype=torch.int16, device="cuda")
    ex = torch.full((n,), -12345, dtype=torch.int32, device="cuda")
    st = torch.cuda.current_stream().cuda_stream
    rc = orth.split_slice_dev(m, n, buf.data_ptr(), ld, planes, dig.data_ptr(), ex.data_ptr(), st)
    assert rc == 0
    torch.cuda.synchronize()
    got = dig.cpu().numpy().view(np.uint16).reshape(planes, nrc, n, 64)
    return got, ex.cpu().numpy()


@pytest.mark.parametrize("m,n,ld,planes", [
    (1000, 19, 1000, 7),        # 16-byte row pairs; partial tile, chunk and column group
    (1000, 19, 1000, 6),
    (777, 21, 779, 7),          # odd m, odd ld: single loads
    (131075, 40, 131076, 7),    # larger, even ld
    (64, 16, 64, 7),            # one chunk, half a tile
])
def test_slice_matches_digit_format(lib, m, n, ld, planes):
    torch = pytest.importorskip("torch")
    X = special_matrix(m, n, seed=m + n)
    want, e_want, _ = digits_reference(X, planes)
    got, e_got = run_slice(torch, X, planes, ld)
    assert np.array_equal(e_got, e_want)
    bad = np.argwhere(got != want)
    assert bad.size == 0, f"{len(bad)} digits differ, first at (plane, chunk, col, row) {bad[0].tolist()}"


def test_digits_reconstruct_the_fixed_point(lib):
    """The digits of every finite normal value give V back, and V 2^(e-55) is within
    half a unit of the 56-bit fixed point of x."""
    torch = pytest.importorskip("torch")
    m, n = 4096, 8
    rng = np.random.default_rng(3)
    X = rng.standard_normal((m, n)) * np.exp2(rng.integers(-8, 8, n))[None, :]
    got, e = run_slice(torch, X, 7, m)
    bf = got.transpose(0, 1, 3, 2).reshape(7, -1, n)[:, :m, :]
    d = (bf.astype(np.uint32) << 16).view(np.float32).astype(np.int64)
    V = np.zeros((m, n), dtype=np.int64)
    for i in range(7):
        V = V * 256 + d[i]
    approx = V.astype(np.float64) * np.exp2(e[None, :].astype(np.float64) - 55.0)
    assert np.all(np.abs(approx - X) <= np.exp2(e[None, :].astype(np.float64) - 56.0))
    assert np.all(np.abs(d[1:]) <= 128) and np.all(np.abs(d[0]) <= 128)

