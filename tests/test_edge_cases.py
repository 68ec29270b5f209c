"""Edge cases and input errors of the C ABI, each turned into a status code and a
message (the reference throws std::runtime_error for these), with the context usable
afterwards.  The host-only entry points are tested without a GPU."""
import ctypes as C

import numpy as np
import pytest

from svfsiplus_gb300 import api, vtkio
from svfsiplus_gb300.mesh import named_pipe


# ---- host-only ---------------------------------------------------------------------
def test_lhsa_isolated_node_and_bad_ids():
    """lhsa (lhsa.cpp:354-356) rejects a node no element holds, and ids out of range."""
    ien = np.array([[0, 1, 2, 3]], dtype=np.int32)
    rowPtr = np.zeros(6, dtype=np.int32)
    nnz = C.c_longlong()
    rc = api.lib().svgpu_lhsa(5, 1, 4, ien.ctypes.data_as(C.c_void_p), rowPtr.ctypes.data_as(C.c_void_p), None,
                              C.byref(nnz))
    assert rc == api.lib().svgpu_lhsa(4, 1, 4, np.array([[0, 1, 2, 9]], np.int32).ctypes.data_as(C.c_void_p),
                                      rowPtr.ctypes.data_as(C.c_void_p), None, C.byref(nnz)) == -1
    rowPtr, colPtr = api.csr_pattern(4, ien)
    assert list(rowPtr) == [0, 4, 8, 12, 16] and colPtr.size == 16


def test_csr_of_ragged_mesh_matches_numpy():
    """A mesh whose rows have very different lengths (a fan of tets around one node)."""
    n = 40
    ien = np.array([[0, i, i + 1, n + 1 + (i % 3)] for i in range(1, n)], dtype=np.int32)
    nNo = n + 4
    rowPtr, colPtr = api.csr_pattern(nNo, ien)
    for r in range(nNo):
        cols = sorted({int(c) for e in ien if r in e for c in e})
        assert list(colPtr[rowPtr[r]:rowPtr[r + 1]]) == cols


def test_restart_truncated_file(tmp_path):
    st = api.restart_stamp(1, 10, 4, False)
    p = tmp_path / "short.bin"
    api.write_restart(p, st, 1, 0.1, [1.0], np.ones((10, 4)), np.ones((10, 4)))
    data = open(p, "rb").read()
    open(p, "wb").write(data[:-8])
    with pytest.raises(RuntimeError, match="too short"):
        api.read_restart(p, st)


def test_write_vtu_rejects_bad_connectivity(tmp_path):
    m = named_pipe("tiny")
    ien = m.ien.copy()
    ien[0, 0] = m.nNo
    with pytest.raises(RuntimeError):
        vtkio.write_vtu(str(tmp_path / "bad.vtu"), m.x, ien, {})


def test_rcr_integrate_rejects_zero_capacitance():
    xn, P = C.c_double(), C.c_double()
    rc = api.lib().svgpu_rcr_integrate(*(C.c_double(v) for v in (121.0, 0.0, 1212.0, 0.0, 1e-3, 0.0, 0.0, 1.0)),
                                       C.byref(xn), C.byref(P))
    assert rc == -1


# ---- on the GPU --------------------------------------------------------------------
def _ctx(m, nfaces=2):
    rowPtr, colPtr = api.csr_pattern(m.nNo, m.ien)
    ctx = api.Context(0)
    ctx.fsils_lhs_create(m.nNo, rowPtr, colPtr, nfaces)
    return ctx, rowPtr, colPtr


@pytest.mark.gpu
def test_bc_create_errors_keep_the_context():
    """fsils_bc_create's own checks (bc.cpp:52-60) and a node out of range."""
    m = named_pipe("tiny")
    ctx, rowPtr, colPtr = _ctx(m)
    with pytest.raises(RuntimeError, match="faIn is exceeding lhs structure maximum number of faces"):
        ctx.fsils_bc_create(2, m.faces["inlet"].gN, 3, api.BC_TYPE_Dir)
    with pytest.raises(RuntimeError, match="faIn is smaller than zero"):
        ctx.fsils_bc_create(-1, m.faces["inlet"].gN, 3, api.BC_TYPE_Dir)
    with pytest.raises(RuntimeError, match="node out of range"):
        ctx.fsils_bc_create(0, np.array([m.nNo], np.int32), 3, api.BC_TYPE_Dir)
    ctx.fsils_bc_create(0, m.faces["inlet"].gN, 3, api.BC_TYPE_Dir)
    ctx.fsils_bc_create(1, np.zeros(0, np.int32), 3, api.BC_TYPE_Dir)  # an empty face is allowed
    ctx.fsils_ls_create(api.LS_TYPE_GMRES, 1e-8, 1e-17, 10, 20)
    ctx.close()


@pytest.mark.gpu
def test_zero_residual_returns_at_once():
    """gmres_v's early return (gmres.cpp:489-495): ||R|| <= absTol leaves R as it is,
    no iteration."""
    m = named_pipe("tiny")
    ctx, rowPtr, colPtr = _ctx(m, 0)
    ctx.fsils_ls_create(api.LS_TYPE_GMRES, 1e-8, 1e-17, 10, 20)
    rng = np.random.default_rng(0)
    Val = rng.standard_normal((colPtr.size, 16))
    R = np.zeros((m.nNo, 4))
    st = ctx.fsils_solve(4, R, Val, api.PREC_FSILS)
    assert st.itr == 0 and not np.any(R) and st.iNorm == 0.0
    ctx.close()


@pytest.mark.gpu
def test_coupled_face_needs_gmres():
    """A coupled (resistance) Neumann face in a CG solve is refused, not ignored."""
    m = named_pipe("tiny")
    ctx, rowPtr, colPtr = _ctx(m, 1)
    ctx.fsils_bc_create(0, m.faces["outlet"].gN, 3, api.BC_TYPE_Neu, np.ones((m.faces["outlet"].gN.size, 3)))
    ctx.fsils_ls_create(api.LS_TYPE_CG, 1e-6, 1e-17, 100, -1)
    rng = np.random.default_rng(1)
    K = rng.standard_normal((colPtr.size, 9))
    with pytest.raises(RuntimeError, match="coupled Neumann faces need GMRES"):
        ctx.fsils_solve(3, rng.standard_normal((m.nNo, 3)), K, api.PREC_FSILS, incL=np.ones(1, np.int32),
                        res=np.array([5.0]))
    # the context still solves: identity diagonal blocks, CG in one iteration
    K = np.zeros((colPtr.size, 9))
    for r in range(m.nNo):
        k = rowPtr[r] + int(np.searchsorted(colPtr[rowPtr[r]:rowPtr[r + 1]], r))
        K[k] = np.eye(3).ravel()
    b = rng.standard_normal((m.nNo, 3))
    x = b.copy()
    st = ctx.fsils_solve(3, x, K, api.PREC_FSILS, incL=np.ones(1, np.int32), res=np.array([0.0]))
    assert st.suc == 1 and np.allclose(x, b)
    ctx.close()


@pytest.mark.gpu
def test_misaligned_device_array_rejected():
    import torch
    m = named_pipe("tiny")
    ctx, rowPtr, colPtr = _ctx(m, 0)
    ctx.fsils_ls_create(api.LS_TYPE_GMRES, 1e-8, 1e-17, 10, 20)
    buf = torch.zeros(4 * m.nNo + 1, dtype=torch.float64, device="cuda")
    Val = torch.zeros(colPtr.size * 16, dtype=torch.float64, device="cuda")
    R = buf[1:]  # 8 bytes past a 256-byte boundary
    with pytest.raises(RuntimeError, match="16-byte aligned"):
        ctx.fsils_solve(4, R, Val, api.PREC_FSILS)
    ctx.close()


@pytest.mark.gpu
def test_fsi_step_without_domains_is_refused():
    m = named_pipe("fsi_tiny")
    ctx, rowPtr, colPtr = _ctx(m, 7)
    ctx.fsils_ls_create(api.LS_TYPE_GMRES, 1e-8, 1e-17, 10, 20)
    ctx.mesh_create(m.x, m.ien)
    opts = api.FsiOpts()
    for q in range(2):
        opts.maxItr[q], opts.lsType[q] = 1, api.LS_TYPE_GMRES
    incl = np.ones(7, np.int32)
    opts.incL[0] = opts.incL[1] = incl.ctypes.data
    opts.outletFace = -1
    z = np.zeros((m.nNo, 7))
    with pytest.raises(RuntimeError, match="mesh_domains"):
        ctx.fsi_step(api.fsi_props(), opts, (np.zeros(0), np.zeros((0, 3)), np.zeros((0, 3))),
                     (np.zeros(0), np.zeros((0, 3)), np.zeros((0, 3))), z, z, z, z.copy(), z.copy(), z.copy(),
                     [0.0, 0.0], [0.0, 0.0])
    ctx.close()


@pytest.mark.gpu
def test_history_and_guess_options_checked():
    """The history slot and the guess threshold are range-checked; a cleared history
    gives no initial guess (x0_rel 0) and the solve still converges."""
    m = named_pipe("tiny")
    ctx, rowPtr, colPtr = _ctx(m, 0)
    ctx.fsils_ls_create(api.LS_TYPE_GMRES, 1e-8, 1e-17, 10, 20)
    with pytest.raises(RuntimeError, match="history_slot"):
        ctx.history_slot(16)
    with pytest.raises(RuntimeError, match="history_slot"):
        ctx.history_slot(-2)
    assert api.lib().svgpu_guess_options(ctx._h, api.C.c_double(0.0)) != api.SVGPU_OK
    assert api.lib().svgpu_guess_options(ctx._h, api.C.c_double(1.5)) != api.SVGPU_OK
    assert api.lib().svgpu_guess_options(ctx._h, api.C.c_double(0.5)) == api.SVGPU_OK
    ctx.history_slot(0)
    ctx.history_clear()
    assert ctx.guess_stats == (0, 0, 0)
    ctx.close()


@pytest.mark.gpu
def test_pinned_host_arrays():
    """Page-locked host arrays (svgpu_host_alloc) start at zero, keep their data, and
    are freed with their last view."""
    import gc
    a = api.pinned_zeros((1000, 4))
    assert a.shape == (1000, 4) and not a.any()
    a[:] = 3.0
    v = a[10:20]
    del a
    gc.collect()
    assert (v == 3.0).all()
    del v
    gc.collect()
    assert api.lib().svgpu_host_free(None) == api.SVGPU_OK
