"""Restart files in the reference's binary layout (output::write_restart,
output.cpp:202-372; init_from_bin, initialize.cpp:78-245), host-only.

Golden: the restart file the compiled reference itself wrote at the end of three golden
runs (tests/golden/ref_*.npz, key restart_bin): the fluid pipe, the fluid pipe with an
RCR outlet (a 0D state in the file) and the coupled FSI pipe (two equations, tDof 7,
dFlag).  The library writes the same bytes from the same state, except the CPU-seconds
field of the header, and reads the reference's files back exactly.
"""
import os

import numpy as np
import pytest

from svfsiplus_gb300 import api

CPU_FIELD = slice(40, 48)  # stamp (28 B) + cTS (4 B) + time (8 B), then the CPU seconds


def _log_rows(g):
    rows = []
    for line in str(g["log"]).splitlines():
        t = line.split()
        if t and t[0] == "step":
            rows.append({k: float(v) for k, v in zip(t[0::2], t[1::2])})
    return rows


def _case(golden, name):
    g = golden(name)
    ps = eval(str(g["params"]))
    n = ps["n_steps"]
    t = 0.0
    for _ in range(n):  # time accumulates as main.cpp does it (time = time + dt)
        t += ps["dt"]
    rows = _log_rows(g)
    if name == "fsi_run_small":
        iNorm = [next(r["iNorm"] for r in rows if r["eq"] == q) for q in (0, 1)]
        Y, A, D = g[f"Yn_{n}"], g[f"An_{n}"], g[f"Dn_{n}"]
        stamp = api.restart_stamp(2, Y.shape[0], 7, True)
        xn = None
    else:
        iNorm = [rows[0]["iNorm"]]
        Y, A, D = g[f"Yn_{n}"], g[f"An_{n}"], None
        xn = None
        nX = 0
        if ps.get("rcr") == 1:  # the 0D state after the last set_bc_cpl of the run
            nX = 1
            xo = ps["rcr_Xo"]
            for k, r in enumerate(rows):
                x, _ = api.rcr_integrate(ps["rcr_Rp"], ps["rcr_C"], ps["rcr_Rd"], ps["rcr_Pd"], ps["dt"], xo,
                                         r["Qo"], r["Qn"])
                if k + 1 < len(rows) and rows[k + 1]["step"] != r["step"]:
                    xo = x
            xn = x
        stamp = api.restart_stamp(1, Y.shape[0], 4, False, nX=nX)
    return g, stamp, n, t, iNorm, Y, A, D, xn


@pytest.mark.parametrize("name", ["small", "small_rcr", "fsi_run_small"])
def test_write_restart_matches_reference_bytes(golden, tmp_path, name):
    g, stamp, n, t, iNorm, Y, A, D, xn = _case(golden, name)
    path = tmp_path / "stFile_last.bin"
    api.write_restart(path, stamp, n, t, iNorm, Y, A, Dn=D, xn=xn)
    ours = np.fromfile(path, dtype=np.uint8)
    ref = g["restart_bin"]
    assert ours.size == ref.size
    mask = np.ones(ref.size, bool)
    mask[CPU_FIELD] = False
    assert np.array_equal(ours[mask], ref[mask])


@pytest.mark.parametrize("name", ["small", "small_rcr", "fsi_run_small"])
def test_read_reference_restart(golden, tmp_path, name):
    g, stamp, n, t, iNorm, Y, A, D, xn = _case(golden, name)
    path = tmp_path / "ref.bin"
    g["restart_bin"].tofile(path)
    r = api.read_restart(path, stamp)
    assert r["cTS"] == n and r["time"] == t
    assert np.array_equal(r["iNorm"], np.asarray(iNorm))
    assert np.array_equal(r["Yo"], Y) and np.array_equal(r["Ao"], A)
    if D is not None:
        assert np.array_equal(r["Do"], D)
    if xn is not None:
        assert r["xo"][0] == xn


def test_read_restart_rejects_other_mesh(golden, tmp_path):
    """A file of another mesh fails with the reference's message."""
    g, stamp, *_ = _case(golden, "small")
    path = tmp_path / "ref.bin"
    g["restart_bin"].tofile(path)
    other = stamp.copy()
    other[3] += 1
    with pytest.raises(RuntimeError, match="The number of nodes"):
        api.read_restart(path, other)
    assert os.path.exists(path)


@pytest.mark.gpu
def test_gpu_restart_continues_bitwise(golden, tmp_path):
    """Two steps, a restart file, a fresh solver that reads it and takes the third step:
    the same fields as three steps in one run, bit for bit (the GPU path is
    deterministic), with the RCR outlet's 0D state carried in the file."""
    g = golden("small_rcr")
    ps = eval(str(g["params"]))
    from svfsiplus_gb300.mesh import named_pipe
    m = named_pipe("small")
    rcr = dict(Rp=ps["rcr_Rp"], C=ps["rcr_C"], Rd=ps["rcr_Rd"], Pd=ps["rcr_Pd"], Xo=ps["rcr_Xo"])

    def solver():
        return api.PipeFluidSolver(m, sD=50, mItr=100, relTol=1e-8, absTol=1e-17, rcr=rcr)

    a = solver()
    for _ in range(3):
        a.step(ps["u_mean"], ps["u_amp"], ps["u_freq"])
    b = solver()
    for _ in range(2):
        b.step(ps["u_mean"], ps["u_amp"], ps["u_freq"])
    path = tmp_path / "stFile_last.bin"
    b.save_restart(path)
    b.ctx.close()
    c = solver()
    c.load_restart(path)
    assert c.cTS == 2
    c.step(ps["u_mean"], ps["u_amp"], ps["u_freq"])
    assert np.array_equal(c.Yn, a.Yn) and np.array_equal(c.An, a.An)
    assert c.ctx.rcr_state()["P"] == a.ctx.rcr_state()["P"]
    a.ctx.close()
    c.ctx.close()
