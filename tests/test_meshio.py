"""Mesh front end (CPU): OBJ and Mitsuba serialized loaders against the
reference's own ParseObj / LoadSerialized (fixture cfgM_mesh, made by the
reference harness on drmlt/scenegen.py:config_meshes), plus the format's
round trip and error behaviour."""
from __future__ import annotations

import gzip
import json
import os

import numpy as np
import pytest

from helpers import GOLDEN
from drmlt import meshio, scenegen
from drmlt import scene as dscene


@pytest.fixture(scope="module")
def mesh_scene(tmp_path_factory):
    d = str(tmp_path_factory.mktemp("meshes"))
    return d, dscene.load_scene(scenegen.config_meshes(d))


def _fixture():
    with gzip.open(os.path.join(GOLDEN, "cfgM_mesh.jsonl.gz"), "rt") as f:
        return [json.loads(line) for line in f]


def test_meshes_match_reference_loaders(mesh_scene):
    """Per shape, every triangle's world-space corner positions and shading
    normals as the reference loaded them (positions within float rounding of
    the transform, normals within 1e-5 -- including the angle weights of the
    computed vertex normals)."""
    _, sd = mesh_scene
    recs = _fixture()
    assert [r["shape"] for r in recs] == list(range(6))
    for r in recs:
        i = r["shape"]
        a, n = int(sd.shape_first_tri[i]), int(sd.shape_num_tris[i])
        p = np.asarray(r["p"], np.float64).reshape(-1, 3, 3)
        nn = np.asarray(r["n"], np.float64).reshape(-1, 3, 3)
        assert p.shape[0] == n, i
        np.testing.assert_allclose(sd.positions[a:a + n], p, atol=2e-6, rtol=0, err_msg="shape %d" % i)
        np.testing.assert_allclose(sd.normals[a:a + n], nn, atol=1e-5, rtol=0, err_msg="shape %d" % i)


def test_reference_angle_weight_is_pinned(mesh_scene):
    """The fixture tells the reference's obtuse-corner weight (pi - 2) * asin(|u+v|/2)
    from the geometric angle: with arccos weights shapes 0, 3 and 5 miss by > 0.05."""
    _, sd = mesh_scene
    rec = _fixture()[3]
    gV = np.asarray(rec["p"], np.float64).reshape(-1, 3)
    keys, F = np.unique(gV.round(6), axis=0, return_inverse=True)
    P = gV[[np.flatnonzero(F == k)[0] for k in range(len(keys))]]
    F = F.reshape(-1, 3)
    ours = meshio.compute_vertex_normals(P, F)[F]
    fn = np.cross(P[F[:, 1]] - P[F[:, 0]], P[F[:, 2]] - P[F[:, 0]])
    ok = np.linalg.norm(fn, axis=1) > 0
    geo = np.zeros_like(P)
    for i in range(3):
        a = P[F[ok, (i + 1) % 3]] - P[F[ok, i]]
        b = P[F[ok, (i + 2) % 3]] - P[F[ok, i]]
        ang = np.arccos(np.clip(np.einsum("ij,ij->i", a, b) / np.linalg.norm(a, axis=1) / np.linalg.norm(b, axis=1),
                                -1, 1))
        np.add.at(geo, F[ok, i], fn[ok] / np.linalg.norm(fn[ok], axis=1, keepdims=True) * ang[:, None])
    geo = (geo / np.linalg.norm(geo, axis=1, keepdims=True))[F]
    ref = np.asarray(rec["n"], np.float64).reshape(-1, 3, 3)
    assert np.abs(ours - ref).max() < 1e-5
    assert np.abs(geo - ref).max() > 0.05


@pytest.mark.parametrize("version,double", [(4, False), (4, True), (3, False), (3, True)])
def test_serialized_round_trip(tmp_path, version, double):
    rng = np.random.default_rng(version * 2 + double)
    meshes = []
    for k in range(3):
        V = rng.normal(size=(20 + k, 3))
        F = rng.integers(0, len(V), (30, 3))
        meshes.append(dict(positions=V, indices=F, normals=rng.normal(size=V.shape) if k != 1 else None,
                           uvs=rng.uniform(size=(len(V), 2)) if k == 2 else None, name="m%d" % k))
    fn = str(tmp_path / "m.serialized")
    meshio.write_serialized(fn, meshes, version=version, double=double)
    tol = 0 if double else 1e-6
    M = np.diag([2.0, 0.5, 1.0, 1.0])
    M[:3, 3] = [0.1, 0.2, 0.3]
    for k, m in enumerate(meshes):
        p, n = meshio.load_serialized(fn, k, M)
        V, F = m["positions"], m["indices"]
        np.testing.assert_allclose(p, (V * [2.0, 0.5, 1.0] + [0.1, 0.2, 0.3])[F], atol=tol * 4 + 1e-6)
        if m["normals"] is not None:
            np.testing.assert_allclose(n, (m["normals"] * [0.5, 2.0, 1.0])[F], atol=tol * 4 + 1e-6)
        else:
            Vw = V * [2.0, 0.5, 1.0] + [0.1, 0.2, 0.3]
            np.testing.assert_allclose(n, meshio.compute_vertex_normals(Vw, F)[F], atol=1e-5)


def test_loader_errors(tmp_path):
    fn = str(tmp_path / "m.serialized")
    meshio.write_serialized(fn, [dict(positions=np.eye(3), indices=[[0, 1, 2]])], version=4)
    with pytest.raises(ValueError, match="out of range"):
        meshio.load_serialized(fn, 1, np.eye(4))
    with open(fn, "rb") as f:
        data = f.read()
    bad = str(tmp_path / "bad.serialized")
    with open(bad, "wb") as f:
        f.write(b"\x00\x00" + data[2:])
    with pytest.raises(ValueError, match="not a serialized"):
        meshio.load_serialized(bad, 0, np.eye(4))
    obj = tmp_path / "ngon.obj"
    obj.write_text("v 0 0 0\nv 1 0 0\nv 1 1 0\nv 0 1 0\nv 0 2 0\nf 1 2 3 4 5\n")
    with pytest.raises(ValueError, match="n-gon"):
        meshio.load_obj(str(obj), np.eye(4))
    obj.write_text("v 0 0 0\nv 1 0 0\nv 1 1 0\nv 0 1 0\nvn 0 0 1\nf 1//1 2//1 3//1\nf 1 3 4\n")
    with pytest.raises(ValueError, match="mix"):
        meshio.load_obj(str(obj), np.eye(4))


def test_animated_transform_rejected(mesh_scene, tmp_path):
    d, _ = mesh_scene
    xml = open(os.path.join(d, "scene.xml")).read().replace(
        '<transform name="toWorld"><scale x="2" y="0.5" z="1"/><translate x="0.1" y="0" z="-0.3"/></transform>',
        '<animation name="toWorld"><transform time="0"/><transform time="1"/></animation>')
    path = os.path.join(d, "animated.xml")
    with open(path, "w") as f:
        f.write(xml)
    with pytest.raises(ValueError, match="animated"):
        dscene.load_scene(path)
