"""svgpu_fsils_dot_noalloc: the dot product for callers that must not allocate device
memory (a host program whose device memory belongs to another allocator or a fixed
budget).  Called through the C ABI, its result is checked against the existing
entry point that computes the same reduction with allocated scratch: fsils_solve
without preconditioning reports iNorm = ||R|| (RI.iNorm, gmres.cpp:481-483).
Tolerance 1e-12 relative, as the FP64 parity tests use; two calls in a row."""
import ctypes as C

import numpy as np
import pytest

from svfsiplus_gb300 import api
from svfsiplus_gb300.mesh import named_pipe

pytestmark = pytest.mark.gpu


def _dot_noalloc(dof, nNo, U, V, stream=None):
    out = C.c_double(0.0)
    rc = api.lib().svgpu_fsils_dot_noalloc(int(dof), int(nNo), C.c_void_p(U.data_ptr()), C.c_void_p(V.data_ptr()),
                                           C.byref(out), stream)
    return rc, out.value


def test_noalloc_dot_matches_fsils_solve_norm():
    import torch
    m = named_pipe("small")
    rowPtr, colPtr = api.csr_pattern(m.nNo, m.ien)
    ctx = api.Context(0)
    ctx.fsils_lhs_create(m.nNo, rowPtr, colPtr, 0)
    ctx.fsils_ls_create(api.LS_TYPE_GMRES, 1e-2, 1e-17, 1, 10)
    rng = np.random.default_rng(11)
    for call in range(2):
        R = rng.standard_normal((m.nNo, 4))
        Val = rng.standard_normal((colPtr.size, 16))  # any matrix: only iNorm = ||R|| is compared
        st = ctx.fsils_solve(4, R.copy(), Val, api.PREC_NONE, incL=None, res=None)
        dR = torch.from_numpy(R).cuda()
        rc, d = _dot_noalloc(4, m.nNo, dR, dR)
        assert rc == 0
        assert abs(np.sqrt(d) - st.iNorm) <= 1e-12 * st.iNorm, (call, np.sqrt(d), st.iNorm)
        V = torch.from_numpy(rng.standard_normal((m.nNo, 4))).cuda()
        rc, d2 = _dot_noalloc(4, m.nNo, dR, V)
        assert rc == 0 and abs(d2 - float((dR * V).sum())) <= 1e-12 * float(dR.norm() * V.norm())


def test_noalloc_dot_device_result_and_limits():
    import torch
    n = 3 * 1000003  # several partial sums, a ragged last one
    U = torch.randn(n, dtype=torch.float64, device="cuda")
    V = torch.randn(n, dtype=torch.float64, device="cuda")
    res = torch.zeros(1, dtype=torch.float64, device="cuda")
    for _ in range(2):
        rc = api.lib().svgpu_fsils_dot_noalloc(3, 1000003, C.c_void_p(U.data_ptr()), C.c_void_p(V.data_ptr()),
                                               C.c_void_p(res.data_ptr()), None)
        torch.cuda.synchronize()
        assert rc == 0
        ref = float((U * V).sum())
        assert abs(float(res.item()) - ref) <= 1e-12 * float(U.norm() * V.norm())
    # beyond the fixed scratch: rejected, nothing launched
    rc = api.lib().svgpu_fsils_dot_noalloc(4, 4 * 1024 * 1024 + 1, C.c_void_p(U.data_ptr()),
                                           C.c_void_p(V.data_ptr()), C.c_void_p(res.data_ptr()), None)
    assert rc == -7
    # host vectors are rejected (the entry point copies nothing in)
    h = np.zeros(8)
    out = C.c_double()
    rc = api.lib().svgpu_fsils_dot_noalloc(4, 2, h.ctypes.data_as(C.c_void_p), h.ctypes.data_as(C.c_void_p),
                                           C.byref(out), None)
    assert rc == -1
