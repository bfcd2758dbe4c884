"""Emulated FP64 GEMM (Ozaki slices and the modular scheme on bf16 tensor
cores) parity.

1. Exactness: integer operands are represented exactly by their slices, so
   the result must equal the exact integer product bit for bit -- including
   the worst case where every digit is +-255 and each 256-deep FP32
   accumulation reaches its largest value (256*255^2 < 2^24), over several
   4096-deep K segments.
2. Accuracy against a double-double reference on uniform(-1,1) and
   exponent-spread operands U*2^E: normwise error
   ||C - Cref||_max / ||G||_max, G = |alpha||A||B| + |beta||C| (the DMMCH
   denominator), bounded by 8*eps for 7 slices (56 bits) on e = 0 operands.
3. The DGEMM contract: transposes, padded leading dimensions, alpha/beta,
   beta = 0 overwriting NaN, and Inf/NaN inputs propagating.
4. The modular scheme (automatic mode): bit for bit the exact integer product
   of the t-bit cut operands, rounded once (a restatement in Python
   integers), over transposes and K segments; the per-tile choice between the
   schemes follows the bounds restated in numpy.
"""
from __future__ import annotations

import math

import numpy as np
import pytest

from conftest import EPS, dmmch_ratio
from test_modular_model import MOD_COUNT, mod_bits

from openblas_gb300 import workloads as W

pytestmark = pytest.mark.gpu


@pytest.fixture
def emulated(gblib):
    gblib.gb_set_dgemm_mode(1)
    yield gblib
    gblib.gb_set_dgemm_mode(0)


def _int_matrix(seed, shape, lo=-127, hi=127):
    return np.asfortranarray(W.randint(seed, shape, lo, hi).astype(np.float64))


# (2200, 3000, 200): 18 m-tiles, so the tile order's last group is a ragged 2
@pytest.fixture(params=[1, 0], ids=["modular", "slices"])
def scheme(request, gblib):
    """Automatic mode with the modular scheme allowed (1) or digit slices only (0)."""
    assert gblib.gb_set_ozaki_modular(request.param) == 0
    yield request.param
    gblib.gb_set_ozaki_modular(1)


@pytest.mark.parametrize("m,n,k", [(64, 48, 1000), (300, 520, 2100), (128, 256, 5000),
                                   (2200, 3000, 200)])
def test_integer_operands_exact(F, emulated, gblib, scheme, m, n, k):
    A = _int_matrix(1, (m, k))
    B = _int_matrix(2, (k, n))
    C = np.zeros((m, n), order="F")
    F.dgemm("N", "N", m, n, k, 1.0, A, m, B, k, 0.0, C, m)
    assert gblib.gb_last_ozaki_moduli() == (MOD_COUNT if scheme else 0)
    exact = (A.astype(np.int64) @ B.astype(np.int64)).astype(np.float64)
    assert np.array_equal(C, exact)


def test_worst_case_digits_exact(F, emulated, gblib, scheme):
    """All digits (residues) +-255 with aligned signs: every 256-deep chunk
    sum is 256*65025 (just below 2^24) and every level sum of a 4096-deep
    segment 4096*65025; k = 9000 spans three segments."""
    m, n, k = 130, 260, 9000
    A = np.full((m, k), 255.0, order="F")
    B = np.full((k, n), 255.0, order="F")
    A[::2] = -255.0
    C = np.zeros((m, n), order="F")
    F.dgemm("N", "N", m, n, k, 1.0, A, m, B, k, 0.0, C, m)
    assert gblib.gb_last_ozaki_moduli() == (MOD_COUNT if scheme else 0)
    exact = np.where(np.arange(m)[:, None] % 2 == 0, -1.0, 1.0) * (k * 255.0 * 255.0)
    assert np.array_equal(C, np.broadcast_to(exact, (m, n)))


def test_multi_digit_exact(F, emulated):
    """Operands with several nonzero 8-bit digits (integers below 2^41 with a
    common row scale) are represented exactly by the default automatic form
    (a 55-bit cut for the modular scheme, or up to 8 digit slices), so the
    product is exact up to its final rounding."""
    m, n, k = 96, 96, 300
    A = _int_matrix(3, (m, k), -(2 ** 20), 2 ** 20)
    B = _int_matrix(4, (k, n), -(2 ** 20), 2 ** 20)
    A[:, 0] = 2.0 ** 40  # every row max -> exponent 41; digits span 41 bits
    C = np.zeros((m, n), order="F")
    F.dgemm("N", "N", m, n, k, 1.0, A, m, B, k, 0.0, C, m)
    exact = A.astype(object) @ B.astype(object)
    err = max(abs(float(C[i, j] - exact[i, j])) for i in range(0, m, 7) for j in range(0, n, 5))
    ref_scale = float(np.abs(A).max() * np.abs(B).max() * k)
    assert err <= 2 * EPS * ref_scale


def _normwise(Cg, Cref, G):
    return np.abs(Cg - Cref).max() / G.max()


# 8-bit slices: 7 keep 56 bits (the default), 6 keep 48
@pytest.mark.parametrize("e,slices,bound", [(0, 7, 8), (0, 6, 200), (8, 7, 32), (16, 7, 256),
                                            (0, 8, 8)])
def test_accuracy_vs_double_double(orc, F, emulated, gblib, e, slices, bound):
    m = n = k = 384
    A = W.exponent_spread(10 + e, (m, k), e)
    B = W.exponent_spread(20 + e, (k, n), e)
    C = W.uniform(30, (m, n))
    gblib.gb_set_ozaki_slices(slices)
    try:
        Cg = C.copy(order="F")
        F.dgemm("N", "N", m, n, k, 1.0, A, m, B, k, 0.0, Cg, m)
    finally:
        gblib.gb_set_ozaki_slices(0)
    Cref = C.copy(order="F")
    orc.dgemm_dd("N", "N", m, n, k, 1.0, A, m, B, k, 0.0, Cref, m)
    G = orc.dgemm_absbound("N", "N", m, n, k, 1.0, A, m, B, k, 0.0, C, m)
    # normwise error against ||G||: FP64 level (the native FP64 GEMM has up to k*eps)
    assert _normwise(Cg, Cref, G) <= bound * EPS, _normwise(Cg, Cref, G) / EPS


@pytest.mark.parametrize("ta,tb", [("N", "N"), ("N", "T"), ("T", "N"), ("T", "T")])
def test_transposes_padding_alpha_beta(orc, F, emulated, ta, tb):
    m, n, k = 333, 290, 1111
    A, B, C = W.gemm_operands(70, m, n, k, ta, tb, pad=8)
    C0 = C.copy(order="F")
    F.dgemm(ta, tb, m, n, k, -1.5, A, A.shape[0], B, B.shape[0], 0.5, C, C.shape[0])
    Cref = C0.copy(order="F")
    orc.dgemm_dd(ta, tb, m, n, k, -1.5, A, A.shape[0], B, B.shape[0], 0.5, Cref, C0.shape[0])
    G = orc.dgemm_absbound(ta, tb, m, n, k, -1.5, A, A.shape[0], B, B.shape[0], 0.5, C0,
                           C0.shape[0])
    assert dmmch_ratio(C[:m], Cref[:m], G, k) <= 16
    assert np.array_equal(C[m:], C0[m:])


def test_beta_zero_and_special_values(F, emulated):
    m, n, k = 70, 90, 200
    A = W.uniform(1, (m, k))
    B = W.uniform(2, (k, n))
    C = np.full((m, n), np.nan, order="F")
    F.dgemm("N", "N", m, n, k, 1.0, A, m, B, k, 0.0, C, m)
    assert np.isfinite(C).all()
    A2 = A.copy(order="F")
    A2[5, 17] = np.inf
    A2[9, 3] = np.nan
    C2 = np.zeros((m, n), order="F")
    F.dgemm("N", "N", m, n, k, 1.0, A2, m, B, k, 0.0, C2, m)
    ref = A2 @ B
    assert np.array_equal(np.isnan(C2), np.isnan(ref))
    assert np.array_equal(np.isinf(C2), np.isinf(ref))
    fin = np.isfinite(ref)
    assert np.abs(C2[fin] - ref[fin]).max() <= 1e-12


def test_large_k_segments(orc, F, emulated):
    """K beyond one 16384 segment: segments accumulate into C."""
    m, n, k = 64, 40, 20000
    A = W.uniform(5, (m, k))
    B = W.uniform(6, (k, n))
    C = W.uniform(7, (m, n))
    Cg, Cref = C.copy(order="F"), C.copy(order="F")
    F.dgemm("N", "N", m, n, k, 1.0, A, m, B, k, 1.0, Cg, m)
    orc.dgemm_dd("N", "N", m, n, k, 1.0, A, m, B, k, 1.0, Cref, m)
    G = orc.dgemm_absbound("N", "N", m, n, k, 1.0, A, m, B, k, 1.0, C, m)
    assert dmmch_ratio(Cg, Cref, G, k) <= 16


def test_device_entry_point(orc, gblib):
    torch = pytest.importorskip("torch")
    m, n, k = 256, 256, 1024
    A, B, C = W.gemm_operands(80, m, n, k, "N", "N")
    dA, dB = torch.from_numpy(A.T.copy()).cuda(), torch.from_numpy(B.T.copy()).cuda()
    dC = torch.from_numpy(C.T.copy()).cuda()
    assert gblib.gb_dgemm_emulated_dev(b"N", b"N", m, n, k, 2.0, dA.data_ptr(), m, dB.data_ptr(),
                                       k, -1.0, dC.data_ptr(), m, 8) == 0
    assert gblib.gb_synchronize() == 0
    got = dC.cpu().numpy().T
    Cref = C.copy(order="F")
    orc.dgemm_dd("N", "N", m, n, k, 2.0, A, m, B, k, -1.0, Cref, m)
    G = orc.dgemm_absbound("N", "N", m, n, k, 2.0, A, m, B, k, -1.0, C, m)
    assert dmmch_ratio(got, Cref, G, k) <= 16


def _device_emulated(gblib, ta, tb, m, n, k, alpha, A, B, beta, C):
    torch = pytest.importorskip("torch")
    dA, dB = torch.from_numpy(A.T.copy()).cuda(), torch.from_numpy(B.T.copy()).cuda()
    dC = torch.from_numpy(C.T.copy()).cuda()
    assert gblib.gb_dgemm_emulated_dev(ta.encode(), tb.encode(), m, n, k, alpha, dA.data_ptr(),
                                       A.shape[0], dB.data_ptr(), B.shape[0], beta,
                                       dC.data_ptr(), C.shape[0], 0) == 0  # default slices
    assert gblib.gb_synchronize() == 0
    return dC.cpu().numpy().T


@pytest.mark.parametrize("ta,tb,beta,pad", [("N", "N", 0.0, 0), ("T", "T", 0.5, 8),
                                            ("N", "T", -1.0, 3)])
def test_host_pipelined_equals_single_call(F, emulated, gblib, ta, tb, beta, pad):
    """Host-pointer DGEMM with n >= 6144 runs column block by column block
    with the uploads and downloads overlapping the other blocks' kernels;
    every C(i,j) depends only on row i of op(A) and column j of op(B), so
    the result equals the device-pointer single-call GEMM bit for bit --
    including a ragged last block, padded leading dimensions, beta != 0
    (C uploaded per block) and an Inf in a later block's column."""
    m, n, k = 2100, 6500, 300
    A, B, C = W.gemm_operands(90, m, n, k, ta, tb, pad=pad)
    if tb == "N":
        B[7, 6400] = np.inf
    else:
        B[6400, 7] = np.inf
    ref = _device_emulated(gblib, ta, tb, m, n, k, 1.25, A, B, beta, C)
    F.dgemm(ta, tb, m, n, k, 1.25, A, A.shape[0], B, B.shape[0], beta, C, C.shape[0])
    assert np.array_equal(C, ref, equal_nan=True)
    assert np.isinf(C[:m, 6400]).any()


def test_host_pipelined_several_k_segments(F, emulated, gblib):
    """K beyond one 4096-deep segment on the column-blocked host path: op(A)
    is split again per segment inside each block, and the segments
    accumulate into C; still bit-identical to the single device call."""
    m, n, k = 2048, 6200, 5000
    A, B, C = W.gemm_operands(92, m, n, k, "T", "N", pad=2)
    ref = _device_emulated(gblib, "T", "N", m, n, k, -0.5, A, B, 2.0, C)
    F.dgemm("T", "N", m, n, k, -0.5, A, A.shape[0], B, B.shape[0], 2.0, C, C.shape[0])
    assert np.array_equal(C, ref)


@pytest.mark.parametrize("hard", [False, True])
def test_host_pipelined_planned_blocks(F, emulated, gblib, hard):
    """A shape whose block plan is uneven (one-wave edge blocks of 4 tiles
    at m = 4096, two or three wider blocks between them, a ragged last
    one), op(A) = A^T arriving in eight row blocks prepared one by one:
    still bit-identical to the single device call.  With `hard`, 200
    columns of op(B) in a late block meet a tiny column of op(A) (the
    construction of the per-tile test below), so that block alone needs
    digit slices: op(A)'s digit split then runs for it only."""
    m, n, k = 4096, 8292, 700
    A, B, C = W.gemm_operands(93, m, n, k, "T", "T", pad=1)  # op(A) = A^T: row blocks
    if hard:
        A[0, :] *= 2.0 ** -30
        B[6000:6200, :k] = np.ldexp(W.uniform(94, (200, k)), -40)
        B[6000:6200, 0] = 1.0
    ref = _device_emulated(gblib, "T", "T", m, n, k, 0.75, A, B, -1.5, C)
    F.dgemm("T", "T", m, n, k, 0.75, A, A.shape[0], B, B.shape[0], -1.5, C, C.shape[0])
    assert np.array_equal(C, ref)
    if hard:
        assert (gblib.gb_last_ozaki_moduli(), gblib.gb_last_ozaki_slices()) == (MOD_COUNT, 8)


def test_host_pipelined_nn_row_blocks(F, emulated, gblib):
    """op(A) = A with at least 8192 rows goes up in row blocks of at least 4096
    rows (strided 2D copies of 32 KB runs), each block's exponents and
    residues prepared while the next uploads: here blocks of 4224 and 4076
    rows with a padded lda and beta != 0, bit-identical to the single device
    call."""
    m, n, k = 8300, 6200, 300
    A, B, C = W.gemm_operands(95, m, n, k, "N", "N", pad=3)
    ref = _device_emulated(gblib, "N", "N", m, n, k, -1.25, A, B, 0.5, C)
    F.dgemm("N", "N", m, n, k, -1.25, A, A.shape[0], B, B.shape[0], 0.5, C, C.shape[0])
    assert np.array_equal(C, ref)


def test_host_pipelined_two_engine_segments(F, emulated, gblib):
    """K beyond one 8192-deep engine segment with op(A) = A^T: op(A) goes up
    in K pieces (row blocks need a single segment) and is prepared per
    segment inside the first column block; still bit-identical to the single
    device call."""
    m, n, k = 2048, 6400, 9000
    A, B, C = W.gemm_operands(95, m, n, k, "T", "N")
    ref = _device_emulated(gblib, "T", "N", m, n, k, 1.0, A, B, 0.0, C)
    F.dgemm("T", "N", m, n, k, 1.0, A, A.shape[0], B, B.shape[0], 0.0, C, C.shape[0])
    assert np.array_equal(C, ref)


@pytest.mark.parametrize("ta,slices,hard", [("N", 0, False), ("T", 0, False), ("N", 0, True),
                                             ("T", 7, False)])
def test_syrk_shaped_reuses_op_a(gblib, ta, slices, hard):
    """C = op(A) op(A)^T with op(B) the same matrix: op(B)'s residues and
    digits are op(A)'s rows, which the engine reuses.  The result must equal
    the product with op(B) a separate copy of the same values (split on its
    own) bit for bit -- n = 600 makes op(A)'s plane stride (640 rows) differ
    from op(B)'s (768); `hard` gives some tiles digit slices."""
    torch = pytest.importorskip("torch")
    n, k = 600, 300
    tb = "T" if ta == "N" else "N"
    A = W.uniform(96, (n, k) if ta == "N" else (k, n))
    if hard:  # one tiny column of op(A) against columns of op(B) led by a large entry
        if ta == "N":
            A[:, 0] *= 2.0 ** -30
            A[300:500, 1:] *= 2.0 ** -40
        else:
            A[0, :] *= 2.0 ** -30
            A[1:, 300:500] *= 2.0 ** -40
    A = np.asfortranarray(A)
    ld = A.shape[0]
    dA = torch.from_numpy(A.T.copy()).cuda()
    dB = dA.clone()
    out = []
    for B in (dA, dB):
        dC = torch.zeros((n, n), dtype=torch.float64, device="cuda")
        assert gblib.gb_dgemm_emulated_dev(ta.encode(), tb.encode(), n, n, k, 1.0, dA.data_ptr(), ld,
                                           B.data_ptr(), ld, 0.0, dC.data_ptr(), n, slices) == 0
        assert gblib.gb_synchronize() == 0
        out.append(dC.cpu().numpy())
    assert np.array_equal(out[0], out[1])
    opA = A if ta == "N" else A.T
    assert np.allclose(out[0].T, opA @ opA.T, rtol=0, atol=1e-12 * k)


@pytest.mark.parametrize("m,n,k,engine", [(256, 256, 256, "native"), (512, 512, 512, "emulated"),
                                           (2048, 2048, 32, "native"), (384, 384, 384, "emulated")])
def test_auto_mode_picks_the_faster_engine(gblib, gb_clean, m, n, k, engine):
    """GB_DGEMM_MODE=auto: the emulated GEMM from m n k >= 384^3 with k >= 64
    (the measured crossover), the native one below; the result equals that
    engine's own entry bit for bit."""
    torch = pytest.importorskip("torch")
    g = torch.Generator(device="cuda")
    g.manual_seed(m + k)
    A = torch.rand((k, m), dtype=torch.float64, device="cuda", generator=g) * 2 - 1
    B = torch.rand((n, k), dtype=torch.float64, device="cuda", generator=g) * 2 - 1
    C1 = torch.empty((n, m), dtype=torch.float64, device="cuda")
    C2 = torch.empty_like(C1)
    gblib.gb_set_dgemm_mode(2)
    try:
        assert gblib.gb_dgemm_dev(b"N", b"N", m, n, k, 1.0, A.data_ptr(), m, B.data_ptr(), k, 0.0,
                                  C1.data_ptr(), m) == 0
    finally:
        gblib.gb_set_dgemm_mode(0)
    if engine == "native":
        st = gblib.gb_dgemm_native_dev(b"N", b"N", m, n, k, 1.0, A.data_ptr(), m, B.data_ptr(), k,
                                       0.0, C2.data_ptr(), m)
    else:
        st = gblib.gb_dgemm_emulated_dev(b"N", b"N", m, n, k, 1.0, A.data_ptr(), m, B.data_ptr(),
                                         k, 0.0, C2.data_ptr(), m, 0)
    assert st == 0 and gblib.gb_synchronize() == 0
    assert torch.equal(C1, C2)


def test_host_pipelined_pinned_buffers(emulated, gblib):
    """The same through cblas_dgemm on pinned (page-locked) host buffers."""
    torch = pytest.importorskip("torch")
    from openblas_gb300 import cblas
    ns = cblas()
    m, n, k = 2048, 8192, 512
    A, B, C = W.gemm_operands(91, m, n, k, "N", "N")
    ref = _device_emulated(gblib, "N", "N", m, n, k, 1.0, A, B, 0.0, C)
    Ah = torch.from_numpy(A.T.copy()).pin_memory()
    Bh = torch.from_numpy(B.T.copy()).pin_memory()
    Ch = torch.full((n, m), float("nan"), dtype=torch.float64).pin_memory()
    ns.cblas_dgemm(102, 111, 111, m, n, k, 1.0, Ah.data_ptr(), m, Bh.data_ptr(), k, 0.0,
                   Ch.data_ptr(), m)
    assert np.array_equal(Ch.numpy().T, ref)


def _column_normwise(Cg, Cref, G):
    """max over columns of sum_i |Cg - Cref| / sum_i G: the measure the
    automatic slice count bounds (G = |alpha||A||B| + |beta||C|)."""
    d = np.abs(Cg - Cref).sum(axis=0)
    g = G.sum(axis=0)
    return float((d / np.where(g > 0, g, 1.0)).max())


DROP_C = 7.0 * (1.0 + 1.0 / 128.0)


def _predict_choice(opA, opB, tol=8.0, modular=True):
    """The automatic choice restated (ozaki.cu choose_slices_kernel, with
    FP64 statistics) for a single-segment product op(A) (m x k) op(B)
    (k x n): per 256-column tile,
    the modular scheme if 2^-t max rho2_j meets the budget, else the
    smallest slice count S with 2^-8S max rho_j within it.  Returns whether
    any tile is modular and the largest slice count (0 if none)."""
    m, k = opA.shape
    n = opB.shape[1]
    t = mod_bits(k) if modular else 0
    ra = np.abs(opA).max(axis=1)
    cb = np.abs(opB).max(axis=0)
    e = np.where(ra > 0, np.frexp(ra)[1], 0)
    f = np.where(cb > 0, np.frexp(cb)[1], 0)
    te = np.ldexp(1.0, e[ra > 0]).sum()
    alpha = np.abs(opA).sum(axis=0)
    t1 = alpha.sum()
    s1 = np.abs(opB).sum(axis=0)
    s2 = alpha @ np.abs(opB)
    ok = (cb > 0) & (s2 > 0)
    slack = 1.0 + 1.0 / 256.0                   # covers the device's FP32 statistics
    rho = np.where(ok, slack * (te * s1 + np.ldexp(t1 + DROP_C * k * te, f))
                   / np.where(ok, s2, 1), 0)
    rho2 = np.where(ok, slack * (te * s1 + np.ldexp(t1 + np.ldexp(k * te, -t), f))
                    / np.where(ok, s2, 1), 0)
    budget = tol * 2.0 ** -52 - 3 * 2.0 ** -53
    any_mod, smax = False, 0
    for j0 in range(0, n, 256):
        if t and np.ldexp(rho2[j0:j0 + 256].max(), -t) <= budget:
            any_mod = True
            continue
        S = next((c for c in range(1, 8) if np.ldexp(rho[j0:j0 + 256].max(), -8 * c) <= budget),
                 8)
        smax = max(smax, S)
    return any_mod, smax


# automatic choice (the default): the modular scheme where its bound meets
# the GB_OZAKI_TOL default of 8 eps, else the smallest slice count that does;
# the error stays within 8 eps, column-normwise and normwise
@pytest.mark.parametrize("e", [0, 8, 16])
def test_automatic_slice_count_meets_tolerance(orc, F, emulated, gblib, scheme, e):
    m = n = k = 1024
    A = W.exponent_spread(40 + e, (m, k), e)
    B = W.exponent_spread(50 + e, (k, n), e)
    C = W.uniform(60, (m, n))
    assert gblib.gb_set_ozaki_slices(0) == 0
    Cg = C.copy(order="F")
    F.dgemm("N", "N", m, n, k, 1.0, A, m, B, k, 0.0, Cg, m)
    any_mod, smax = _predict_choice(A, B, modular=bool(scheme))
    if e == 0:
        assert any_mod == bool(scheme) and smax == (0 if scheme else 7)
    assert gblib.gb_last_ozaki_moduli() == (MOD_COUNT if any_mod else 0)
    assert gblib.gb_last_ozaki_slices() == smax
    Cref = C.copy(order="F")
    orc.dgemm_dd("N", "N", m, n, k, 1.0, A, m, B, k, 0.0, Cref, m)
    G = orc.dgemm_absbound("N", "N", m, n, k, 1.0, A, m, B, k, 0.0, C, m)
    assert _column_normwise(Cg, Cref, G) <= 8 * EPS, _column_normwise(Cg, Cref, G) / EPS
    assert _normwise(Cg, Cref, G) <= 8 * EPS, _normwise(Cg, Cref, G) / EPS


def test_automatic_slice_count_per_column_tile(F, emulated, gblib):
    """One 256-column tile of uniform columns next to a tile whose columns
    are dominated by one entry that meets a tiny column of op(A) (so the
    rows' scales are 2^30 above what the products use): each tile gets its
    own scheme.  The uniform tile takes the modular scheme and equals the
    automatic product of its columns alone; the other takes 8 slices and,
    because the first S digits of an 8-digit split are the S-digit split,
    equals the fixed 8-slice result bit for bit.  With the modular scheme
    off, the uniform tile takes 7 slices and equals the fixed 7-slice
    result."""
    m, k = 300, 700
    A = W.uniform(70, (m, k))
    A[:, 0] *= 2.0 ** -30
    hard = np.ldexp(W.uniform(72, (k, 200)), -40)
    hard[0] = 1.0
    B = np.asfortranarray(np.hstack([W.uniform(71, (k, 256)), hard]))
    assert _predict_choice(A, B) == (True, 8)
    assert _predict_choice(A, B, modular=False) == (False, 8)

    def run(s, BB, modular=1):
        assert gblib.gb_set_ozaki_slices(s) == 0
        assert gblib.gb_set_ozaki_modular(modular) == 0
        Cs = np.zeros((m, BB.shape[1]), order="F")
        F.dgemm("N", "N", m, BB.shape[1], k, 1.0, A, m, BB, k, 0.0, Cs, m)
        got = (gblib.gb_last_ozaki_moduli(), gblib.gb_last_ozaki_slices()) if s == 0 else None
        return Cs, got

    try:
        mixed, got = run(0, B)
        assert got == (MOD_COUNT, 8)
        left, got = run(0, np.asfortranarray(B[:, :256]))
        assert got == (MOD_COUNT, 0)
        off, got = run(0, B, modular=0)
        assert got == (0, 8)
        c7, _ = run(7, B)
        c8, _ = run(8, B)
    finally:
        gblib.gb_set_ozaki_slices(0)
        gblib.gb_set_ozaki_modular(1)
    assert np.array_equal(mixed[:, :256], left)
    assert np.array_equal(mixed[:, 256:], c8[:, 256:])
    assert np.array_equal(off[:, :256], c7[:, :256])
    assert np.array_equal(off[:, 256:], c8[:, 256:])


def test_digit_tiles_take_sub_segments(orc, F, emulated, gblib):
    """k = 8192 + 333 with one hard column tile: the modular tiles take the
    8192-deep segments, the digit-slice tile takes them in 4096-deep
    sub-segments (its level sums exact in int32); every column stays within
    the 8 eps tolerance against double-double."""
    m, k = 200, MOD_SEGMENT + 333
    A = W.uniform(84, (m, k))
    A[:, 0] *= 2.0 ** -30
    hard = np.ldexp(W.uniform(85, (k, 100)), -40)
    hard[0] = 1.0
    B = np.asfortranarray(np.hstack([W.uniform(86, (k, 256)), hard]))
    n = B.shape[1]
    C = np.zeros((m, n), order="F")
    F.dgemm("N", "N", m, n, k, 1.0, A, m, B, k, 0.0, C, m)
    assert gblib.gb_last_ozaki_moduli() == MOD_COUNT
    assert gblib.gb_last_ozaki_slices() == 8
    Cref = np.zeros((m, n), order="F")
    orc.dgemm_dd("N", "N", m, n, k, 1.0, A, m, B, k, 0.0, Cref, m)
    G = orc.dgemm_absbound("N", "N", m, n, k, 1.0, A, m, B, k, 0.0, np.zeros((m, n), order="F"), m)
    assert _column_normwise(C[:, :256], Cref[:, :256], G[:, :256]) <= 8 * EPS
    # the hard tile: its 8-slice bound exceeds 8 eps (the rows' scales sit
    # 2^30 above the products that reach it), so only a loose level is asserted
    assert _column_normwise(C[:, 256:], Cref[:, 256:], G[:, 256:]) <= 2.0 ** -16


def _cut(X, e, t, axis):
    """sign(x) trunc(|x| 2^(t - e)) as Python integers, e per row (axis 1)
    or per column (axis 0)."""
    out = np.empty(X.shape, dtype=object)
    for idx, x in np.ndenumerate(X):
        ee = int(e[idx[0]] if axis == 1 else e[idx[1]])
        num, den = abs(float(x)).as_integer_ratio()
        sh = t - ee
        v = (num << sh) // den if sh >= 0 else num // (den << -sh)
        out[idx] = -v if x < 0 else v
    return out


MOD_SEGMENT = 8192


def _modular_expected(opA, opB):
    """alpha = 1, beta = 0: per 8192-deep K segment, C' = A'B' exactly (the
    t-bit cut operands, t from the segment length), C += round(C') 2^(e_i +
    f_j - 2t), the first segment storing."""
    m, k = opA.shape
    n = opB.shape[1]
    t = mod_bits(min(k, MOD_SEGMENT))
    C = np.zeros((m, n))
    for k0 in range(0, k, MOD_SEGMENT):
        Ak, Bk = opA[:, k0:k0 + MOD_SEGMENT], opB[k0:k0 + MOD_SEGMENT, :]
        ra, cb = np.abs(Ak).max(axis=1), np.abs(Bk).max(axis=0)
        e = np.where(ra > 0, np.frexp(ra)[1], 0)
        f = np.where(cb > 0, np.frexp(cb)[1], 0)
        Cp = _cut(Ak, e, t, 1).dot(_cut(Bk, f, t, 0))
        for (i, j), c in np.ndenumerate(Cp):
            v = math.ldexp(float(c), int(e[i] + f[j]) - 2 * t)
            C[i, j] = v if k0 == 0 else C[i, j] + v
    return C


@pytest.mark.parametrize("ta,tb", [("N", "N"), ("N", "T"), ("T", "N"), ("T", "T")])
def test_modular_equals_exact_product_of_cut_operands(F, emulated, gblib, ta, tb):
    """Every element is the exact integer product of the cut operands
    rounded once and scaled: bit for bit, over transposes and padded
    leading dimensions (two column tiles, the second ragged)."""
    m, n, k = 40, 280, 257
    A, B, C = W.gemm_operands(80, m, n, k, ta, tb, pad=5)
    A = np.asfortranarray(A * np.ldexp(1.0, W.randint(81, A.shape, -4, 4)))
    opA = A[:m, :k] if ta == "N" else A[:k, :m].T
    opB = B[:k, :n] if tb == "N" else B[:n, :k].T
    assert _predict_choice(opA, opB)[0]
    Cg = np.full_like(C, np.nan)
    F.dgemm(ta, tb, m, n, k, 1.0, A, A.shape[0], B, B.shape[0], 0.0, Cg, Cg.shape[0])
    assert (gblib.gb_last_ozaki_moduli(), gblib.gb_last_ozaki_slices()) == (MOD_COUNT, 0)
    assert np.array_equal(Cg[:m], _modular_expected(opA, opB))


def test_modular_equals_exact_product_over_k_segments(F, emulated, gblib):
    """k = 8192 + 333: two K segments, each exact and rounded once, the
    second added to the first in FP64."""
    m, n, k = 20, 36, MOD_SEGMENT + 333
    A = W.exponent_spread(82, (m, k), 3)
    B = W.uniform(83, (k, n))
    C = np.zeros((m, n), order="F")
    F.dgemm("N", "N", m, n, k, 1.0, A, m, B, k, 0.0, C, m)
    assert gblib.gb_last_ozaki_moduli() == MOD_COUNT
    assert np.array_equal(C, _modular_expected(A, B))


def test_near_underflow_recombine_matches_native(gblib):
    """Operands near 2^-512 and 2^-500 give C near 2^-1010: the recombine's
    scale alpha * 2^x alone would be subnormal there, so the level total is
    rounded once and scaled by the whole power of two once; the emulated
    result stays within a few eps of |A||B| of the native FP64 one."""
    torch = pytest.importorskip("torch")
    m, n, k = 96, 80, 64
    A = torch.from_numpy(np.ldexp(W.uniform(90, (m, k)), -512).T.copy()).cuda()
    B = torch.from_numpy(np.ldexp(W.uniform(91, (k, n)), -500).T.copy()).cuda()
    Ce = torch.zeros((n, m), dtype=torch.float64, device="cuda")
    Cn = torch.zeros((n, m), dtype=torch.float64, device="cuda")
    G = torch.zeros((n, m), dtype=torch.float64, device="cuda")
    Aa, Ba = A.abs(), B.abs()
    torch.cuda.synchronize()
    for Cx, fn, AA, BB in ((Ce, gblib.gb_dgemm_emulated_dev, A, B),
                           (Cn, gblib.gb_dgemm_native_dev, A, B),
                           (G, gblib.gb_dgemm_native_dev, Aa, Ba)):
        args = [b"N", b"N", m, n, k, 1.0, AA.data_ptr(), m, BB.data_ptr(), k, 0.0, Cx.data_ptr(), m]
        if fn is gblib.gb_dgemm_emulated_dev:
            args.append(0)
        assert fn(*args) == 0
    assert gblib.gb_synchronize() == 0
    torch.cuda.synchronize()
    assert float(G.min()) > 0 and float(G.max()) < 2.0 ** -1000
    err = float(((Ce - Cn).abs() / G).max())
    assert err <= 4 * (k + 2) * EPS, err / EPS


@pytest.mark.parametrize("mode", ["native", "emulated"])
def test_gemm_taller_than_2_20_rows_equals_row_slices(gblib, mode):
    """m = 2^20 + 300 rows (beyond the 2^20 block extent, so the product runs
    block by block over C): every element sees the same row of op(A) and
    column of op(B), so the result equals, bit for bit, the same GEMM called
    on row slices that each fit one block."""
    torch = pytest.importorskip("torch")
    m, n, k = (1 << 20) + 300, 96, 256
    g = torch.Generator(device="cuda")
    g.manual_seed(5)
    A = torch.rand((k, m), dtype=torch.float64, device="cuda", generator=g) * 2 - 1  # A column-major m x k
    B = torch.rand((n, k), dtype=torch.float64, device="cuda", generator=g) * 2 - 1  # B column-major k x n
    C = torch.empty((n, m), dtype=torch.float64, device="cuda")
    R = torch.empty((n, m), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()

    def gemm(rows, r0, out):
        a = A.data_ptr() + 8 * r0
        c = out.data_ptr() + 8 * r0
        if mode == "native":
            return gblib.gb_dgemm_native_dev(b"N", b"N", rows, n, k, 1.0, a, m, B.data_ptr(), k,
                                             0.0, c, m)
        return gblib.gb_dgemm_emulated_dev(b"N", b"N", rows, n, k, 1.0, a, m, B.data_ptr(), k,
                                           0.0, c, m, 7)

    assert gemm(m, 0, C) == 0
    step = 1 << 19
    for r0 in range(0, m, step):
        assert gemm(min(step, m - r0), r0, R) == 0
    assert gblib.gb_synchronize() == 0
    torch.cuda.synchronize()
    assert torch.equal(C, R)
