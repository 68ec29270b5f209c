"""Procedural pipe meshes: conforming, positively oriented, faces owned by tets."""
import numpy as np
import pytest

from svfsiplus_gb300 import api
from svfsiplus_gb300.mesh import named_pipe, make_pipe
from oracle import pyoracle as po


@pytest.mark.parametrize("name", ["tiny", "small", "pipe50k"])
def test_mesh_orientation_and_volume(name):
    m = named_pipe(name)
    x, ien = m.x, m.ien
    d = np.einsum("ij,ij->i", x[ien[:, 0]] - x[ien[:, 3]],
                  np.cross(x[ien[:, 1]] - x[ien[:, 3]], x[ien[:, 2]] - x[ien[:, 3]]))
    assert (d > 0).all()
    vol = d.sum() / 6.0
    assert abs(vol - np.pi * 0.25 * 5.0) / (np.pi * 0.25 * 5.0) < 0.12


def test_mesh_conforming_faces_shared_twice():
    m = named_pipe("small")
    f = np.sort(np.concatenate([m.ien[:, [0, 1, 2]], m.ien[:, [0, 1, 3]], m.ien[:, [0, 2, 3]],
                                m.ien[:, [1, 2, 3]]]), axis=1)
    _, cnt = np.unique(f, axis=0, return_counts=True)
    nb = sum(fa.ien.shape[0] for fa in m.faces.values())
    assert cnt.max() == 2 and (cnt == 1).sum() == nb


def test_face_owner_contains_face():
    m = named_pipe("small")
    for fa in m.faces.values():
        for tri, e in zip(fa.ien, fa.gE):
            assert set(tri) <= set(m.ien[e])


def test_csr_pattern_python_equals_oracle():
    m = named_pipe("small")
    rp, cp = api.csr_pattern(m.nNo, m.ien)
    rp2, cp2 = po.lhsa(m.nNo, m.ien)
    assert np.array_equal(rp, rp2) and np.array_equal(cp, cp2)


def test_perturbed_wall_is_seeded():
    a = make_pipe(4, 2, 4, perturb_modes=8)
    b = make_pipe(4, 2, 4, perturb_modes=8)
    assert np.array_equal(a.x, b.x) and a.params["amp"] == b.params["amp"]
    assert sum(a.params["amp"]) <= 0.1 + 1e-12
