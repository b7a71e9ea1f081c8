"""GPU: the dense complex kernels of the LU, called through the C ABI.

- gbi_tc_cgemm_sub (tcgen05 tensor cores, complex FP32 as a real TF32 GEMM on
  interleaved storage) against a plain PyTorch reference of the same op:
  the three-pass split must carry FP32-level error (<= 2e-6 relative
  Frobenius), the one-pass form TF32-level error (<= 2e-3); shapes include
  ragged edges and sub-matrices with leading dimensions, as in the LU.
- gbi_cgetrf / gbi_zgetrf (tournament-pivoting LU): P A = L U to FP32 / FP64
  rounding, against the factors read back to the host.
The FP32 factorisations are checked in the FP32-accurate three-pass mode
(gb_set_tc_passes(3)); the library's default single pass is covered by the
GMRES tests, which only need a preconditioner.
"""
import ctypes

import numpy as np
import pytest

vp, ci, csz = ctypes.c_void_p, ctypes.c_int, ctypes.c_size_t


def _lib():
    from bem3_emf_b2_gb300 import lib
    L = lib()
    L.gbi_tc_cgemm_sub.argtypes = [ci, ci, ci, vp, csz, vp, csz, vp, csz, ci, vp, vp, vp]
    L.gbi_tc_cgemm_sub.restype = ci
    for f in (L.gbi_cgetrf, L.gbi_zgetrf, L.gbi_cgetrf_simt):
        f.argtypes = [vp, csz, ci, vp, vp, vp]
        f.restype = ci
    return L


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.fixture(autouse=True)
def _three_pass(gb_build):
    from bem3_emf_b2_gb300 import lib
    L = lib()
    L.gb_set_tc_passes.argtypes = [ci]
    L.gb_get_tc_passes.restype = ci
    keep = L.gb_get_tc_passes()
    L.gb_set_tc_passes(3)
    yield
    L.gb_set_tc_passes(keep)


@pytest.mark.gpu
@pytest.mark.parametrize("M,N,K,pad", [(128, 128, 64, 0), (300, 200, 64, 0), (1000, 517, 50, 3), (77, 900, 7, 5),
                                       (1536, 1536, 64, 64)])
def test_tc_cgemm_matches_torch(M, N, K, pad, gb_build):
    import torch
    L = _lib()
    g = torch.Generator().manual_seed(M * 7 + N + K)
    ld = max(K, N) + pad
    big = torch.randn(M + K, ld, 2, generator=g, dtype=torch.float32)
    big = torch.view_as_complex(big).contiguous()
    A = big[K:, :K]            # M x K at row offset K (leading dimension ld)
    B = big[:K, :N]            # K x N
    C0 = torch.randn(M, N + pad, 2, generator=g, dtype=torch.float32)
    C0 = torch.view_as_complex(C0).contiguous()
    ref = C0[:, :N].to(torch.complex128) - A.to(torch.complex128) @ B.to(torch.complex128)
    ref32 = C0[:, :N] - A @ B  # the plain FP32 reference of the same op
    dev = "cuda"
    bigd = big.to(dev)
    for passes, tol in ((3, 2e-6), (1, 2e-3)):
        Cd = C0.to(dev)
        Ad = bigd[K:, :K]
        Bd = bigd[:K, :N]
        rc = L.gbi_tc_cgemm_sub(M, N, K, Ad.data_ptr(), ld, Bd.data_ptr(), ld, Cd.data_ptr(), N + pad, passes, None,
                                None, None)
        assert rc == 0, L.gb_last_error()
        torch.cuda.synchronize()
        out = Cd[:, :N].cpu().to(torch.complex128)
        err = _rel(out.numpy(), ref.numpy())
        err32 = _rel(ref32.to(torch.complex128).numpy(), ref.numpy())
        assert err <= tol, "passes %d: %g (fp32 reference %g)" % (passes, err, err32)
        # the padding columns are untouched
        assert torch.equal(Cd[:, N:].cpu(), C0[:, N:])


def _check_lu(LU, ipiv, A0):
    n = A0.shape[0]
    P = np.arange(n)
    for j in range(n):
        p = int(ipiv[j])
        P[[j, p]] = P[[p, j]]
    Lm = np.tril(LU, -1) + np.eye(n)
    U = np.triu(LU)
    return _rel(Lm @ U, A0[P])


@pytest.mark.gpu
@pytest.mark.parametrize("n", [1, 63, 300, 1000, 2113])
def test_getrf_factors(n, gb_build):
    import torch
    L = _lib()
    rng = np.random.default_rng(n)
    A0 = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    for dt, f, tol in ((torch.complex128, L.gbi_zgetrf, 1e-13), (torch.complex64, L.gbi_cgetrf, 1e-4),
                       (torch.complex64, L.gbi_cgetrf_simt, 1e-4)):
        Ad = torch.tensor(A0, dtype=dt, device="cuda")
        ip = torch.zeros(n, dtype=torch.int64, device="cuda")
        info = torch.zeros(1, dtype=torch.int32, device="cuda")
        assert f(Ad.data_ptr(), n, n, ip.data_ptr(), info.data_ptr(), None) == 0, L.gb_last_error()
        torch.cuda.synchronize()
        assert int(info.item()) == 0
        ipiv = ip.cpu().numpy()
        assert ipiv.min() >= 0 and ipiv.max() < n and np.all(ipiv >= np.arange(n))
        err = _check_lu(Ad.cpu().numpy().astype(np.complex128), ipiv, A0)
        assert err <= tol, "%s n=%d: %g" % (f.__name__, n, err)


@pytest.mark.gpu
@pytest.mark.parametrize("n,nrhs,pad", [(1, 1, 0), (63, 4, 0), (300, 6, 1), (1000, 8, 0), (2113, 4, 1), (4096, 4, 0)])
def test_lu_solve_multi(n, nrhs, pad, gb_build):
    """gbi_csolve_multi / gbi_zsolve_multi (the triangular solves of the
    refinement: gather by the pivot permutation, then one cooperative launch
    per triangle) against numpy's solve with the same factors' matrix; pad
    makes the leading dimension odd (no 16-byte copies of the factor)."""
    import torch
    L = _lib()
    L.gbi_make_perm.argtypes = [vp, ci, vp, vp]
    L.gbi_make_perm.restype = ci
    for f in (L.gbi_csolve_multi, L.gbi_zsolve_multi):
        f.argtypes = [vp, csz, ci, vp, vp, csz, ci, vp, vp]
        f.restype = ci
    rng = np.random.default_rng(n + nrhs)
    A0 = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n)) + 4.0 * np.sqrt(n) * np.eye(n)
    B0 = rng.standard_normal((n, nrhs)) + 1j * rng.standard_normal((n, nrhs))
    ref = np.linalg.solve(A0, B0)
    lda = n + pad
    for dt, getrf, solve, tol in ((torch.complex64, L.gbi_cgetrf, L.gbi_csolve_multi, 1e-4),
                                  (torch.complex128, L.gbi_zgetrf, L.gbi_zsolve_multi, 1e-12)):
        Ap = np.zeros((n, lda), complex)
        Ap[:, :n] = A0
        Ad = torch.tensor(Ap, dtype=dt, device="cuda")
        ip = torch.zeros(n, dtype=torch.int64, device="cuda")
        info = torch.zeros(1, dtype=torch.int32, device="cuda")
        assert getrf(Ad.data_ptr(), lda, n, ip.data_ptr(), info.data_ptr(), None) == 0, L.gb_last_error()
        perm = torch.zeros(n, dtype=torch.int32, device="cuda")
        assert L.gbi_make_perm(ip.data_ptr(), n, perm.data_ptr(), None) == 0
        Xd = torch.tensor(B0, dtype=dt, device="cuda")
        Yd = torch.zeros(n, nrhs, dtype=dt, device="cuda")
        assert solve(Ad.data_ptr(), lda, n, perm.data_ptr(), Xd.data_ptr(), nrhs, nrhs, Yd.data_ptr(), None) == 0, \
            L.gb_last_error()
        torch.cuda.synchronize()
        err = _rel(Yd.cpu().numpy().astype(np.complex128), ref)
        assert err <= tol, "%s n=%d nrhs=%d: %g" % (solve.__name__, n, nrhs, err)


def _butterfly_t(p, n):
    """dense matrix of the depth-2 transposed recursive butterfly U^T for the
    parameters p[2][n] (level 1, level 2), as defined for gbi_rbt_matrix"""
    q = n // 4
    s = 1.0 / np.sqrt(2.0)
    p1, p2 = p[:n], p[n:]

    def level(pairs, pp):
        M = np.zeros((n, n))
        for i in range(q):
            for a, b in pairs:
                ia, ib = i + a * q, i + b * q
                M[ia, ia] = M[ia, ib] = pp[ia] * s
                M[ib, ia] = pp[ib] * s
                M[ib, ib] = -pp[ib] * s
        return M
    L2 = level([(0, 1), (2, 3)], p2)
    L1 = level([(0, 2), (1, 3)], p1)
    return L1 @ L2  # level 2 first


@pytest.mark.gpu
@pytest.mark.parametrize("n", [4, 64, 512])
def test_rbt_transform_matches_dense_model(n, gb_build):
    """gbi_rbt_matrix: A <- U^T A V with U^T, V^T the depth-2 transposed
    butterflies of the parameters (the dense model above); the unpivoted LU
    of the randomised matrix solves the original system as x = V A_r^-1 U^T b."""
    import torch
    L = _lib()
    L.gbi_rbt_matrix.argtypes = [vp, csz, ci, vp, vp, vp]
    L.gbi_rbt_matrix.restype = ci
    L.gbi_cgetrf_nopiv.argtypes = [vp, csz, ci, vp, vp, vp]
    L.gbi_cgetrf_nopiv.restype = ci
    rng = np.random.default_rng(n)
    A0 = (rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))).astype(np.complex64)
    pu = np.exp(rng.uniform(-0.5, 0.5, 2 * n) / 10).astype(np.float32)
    pv = np.exp(rng.uniform(-0.5, 0.5, 2 * n) / 10).astype(np.float32)
    Ut = _butterfly_t(pu.astype(float), n)
    V = _butterfly_t(pv.astype(float), n).T
    ref = Ut @ A0.astype(np.complex128) @ V
    Ad = torch.tensor(A0, device="cuda")
    pud = torch.tensor(pu, device="cuda")
    pvd = torch.tensor(pv, device="cuda")
    assert L.gbi_rbt_matrix(Ad.data_ptr(), n, n, pud.data_ptr(), pvd.data_ptr(), None) == 0, L.gb_last_error()
    torch.cuda.synchronize()
    Ar = Ad.cpu().numpy().astype(np.complex128)
    assert _rel(Ar, ref) <= 2e-6
    ip = torch.zeros(n, dtype=torch.int64, device="cuda")
    info = torch.zeros(1, dtype=torch.int32, device="cuda")
    assert L.gbi_cgetrf_nopiv(Ad.data_ptr(), n, n, ip.data_ptr(), info.data_ptr(), None) == 0, L.gb_last_error()
    torch.cuda.synchronize()
    assert int(info.item()) == 0
    assert np.array_equal(ip.cpu().numpy(), np.arange(n))
    LU = Ad.cpu().numpy().astype(np.complex128)
    Lm = np.tril(LU, -1) + np.eye(n)
    U = np.triu(LU)
    assert _rel(Lm @ U, Ar) <= 1e-4
    b = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    x = V @ np.linalg.solve(Lm @ U, Ut @ b)
    assert _rel(A0.astype(np.complex128) @ x, b) <= 1e-3 * max(1.0, np.linalg.cond(A0) / 1e3)


@pytest.mark.gpu
@pytest.mark.parametrize("n,nrhs", [(6, 6), (64, 1), (258, 6), (1536, 6), (1001, 3)])
def test_zgesv_mixed(n, nrhs, gb_build):
    """gbi_zgesv_mixed (the dE/dn, dH/dn solve of the chosen form): FP32
    factors of the butterfly-randomised matrix (n divisible by 4) or with
    tournament pivoting (otherwise) and FP64 refinement to 1e-13: the FP64
    solution of numpy to that level."""
    import torch
    L = _lib()
    L.gbi_zgesv_mixed.argtypes = [vp, ci, vp, ci, vp, vp, vp, vp]
    L.gbi_zgesv_mixed.restype = ci
    rng = np.random.default_rng(n * 3 + nrhs)
    A0 = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n)) + 2.0 * np.sqrt(n) * np.eye(n)
    B0 = rng.standard_normal((n, nrhs)) + 1j * rng.standard_normal((n, nrhs))
    ref = np.linalg.solve(A0, B0)
    Ad = torch.tensor(A0, dtype=torch.complex128, device="cuda")
    Bd = torch.tensor(B0, dtype=torch.complex128, device="cuda")
    Xd = torch.zeros(n, nrhs, dtype=torch.complex128, device="cuda")
    it, rr = ctypes.c_int(), ctypes.c_double()
    assert L.gbi_zgesv_mixed(Ad.data_ptr(), n, Bd.data_ptr(), nrhs, Xd.data_ptr(), ctypes.byref(it), ctypes.byref(rr),
                             None) == 0, L.gb_last_error()
    torch.cuda.synchronize()
    assert rr.value <= 1e-13 and 1 <= it.value <= 8, (it.value, rr.value)
    assert _rel(Xd.cpu().numpy(), ref) <= 1e-11
