"""OBJ/MTL ingest to arrays (or3_mesh_load_obj, or3_mesh_transform): host code,
no GPU.  Pinned against the reference's own Model::ReadFromObj + Transform
(golden tests/golden/obj_ref.npz, and live when the reference is built here).

The reference adds a model's triangles grouped by material in hash-map order;
the ingest keeps file order.  So the comparison is of the two triangle
multisets: vertices, normals, uvs and material (type, colour, ior) per
triangle, to FP64 rounding (the transform's products are evaluated in the
same order; 1e-12 relative).
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN, golden

MESH = os.path.join(GOLDEN, "obj", "mesh.obj")
TRANSFORM = dict(position=(10.0, -5.0, 3.0), scaling=(2.0, 1.0, 0.5), rotation=(0.3, -0.2, 0.7))


def _rows(tri, nrm, uv, mat):
    n = tri.shape[0]
    return np.concatenate([tri.reshape(n, 9), nrm.reshape(n, 9), uv.reshape(n, 6), mat.reshape(n, 5)], axis=1)


def _ours(pkg, path, flip, **tf):
    m = pkg.load_obj(path, flip_v=flip, **tf)
    mats = np.array([[t, c[0], c[1], c[2], ior] for t, c, ior in m["materials"]])
    return _rows(m["vertices"], m["normals"], m["uvs"], mats[m["material"]]), m


def _same_multiset(a, b):
    assert a.shape == b.shape, (a.shape, b.shape)
    ka = a[np.lexsort(np.round(a, 9).T[::-1])]
    kb = b[np.lexsort(np.round(b, 9).T[::-1])]
    np.testing.assert_allclose(ka, kb, rtol=1e-12, atol=1e-12)


@pytest.mark.parametrize("flip", [0, 1])
def test_obj_matches_reference_golden(pkg, flip):
    g = golden("obj_ref.npz")
    ours, m = _ours(pkg, MESH, bool(flip), **TRANSFORM)
    _same_multiset(ours, _rows(g["tri_%d" % flip], g["nrm_%d" % flip], g["uv_%d" % flip], g["mat_%d" % flip]))
    assert m["names"][:4] == ["__default__material__", "red", "glass", "blue"]
    assert m["textures"] == [None] * 4


def _write_big_obj(pkg, path):
    # a level-5 icosphere with uvs and normals in every face form, > 1 MB (multi-threaded parse)
    v, f = pkg.scene.icosphere(5)
    vn = v / np.linalg.norm(v, axis=1, keepdims=True)
    uv = np.stack([np.arctan2(v[:, 2], v[:, 0]) / (2 * np.pi) + 0.5, v[:, 1] * 0.5 + 0.5], 1)
    with open(path, "w") as fh:
        fh.write("# generated\n")
        fh.writelines("v %.9f %.9f %.9f\n" % tuple(p) for p in v * 10)
        fh.writelines("vt %.6f %.6f\n" % tuple(t) for t in uv)
        fh.writelines("vn %.6f %.6f %.6f\n" % tuple(n) for n in vn)
        for i, (a, b, c) in enumerate(f + 1):
            form = i % 4
            if form == 0:
                fh.write("f %d %d %d\n" % (a, b, c))
            elif form == 1:
                fh.write("f %d/%d %d/%d %d/%d\n" % (a, a, b, b, c, c))
            elif form == 2:
                fh.write("f %d/%d/%d %d/%d/%d %d/%d/%d\n" % (a, a, a, b, b, b, c, c, c))
            else:
                fh.write("f %d//%d %d//%d %d//%d\n" % (a, a, b, b, c, c))
    return len(f)


def test_parallel_parse_equals_serial(pkg, tmp_path):
    path = str(tmp_path / "big.obj")
    n = _write_big_obj(pkg, path)
    assert os.path.getsize(path) > (1 << 20)
    a = pkg.load_obj(path, threads=1)
    b = pkg.load_obj(path, threads=16)
    assert a["vertices"].shape[0] == n
    for k in ("vertices", "normals", "uvs", "material"):
        np.testing.assert_array_equal(a[k], b[k])


@pytest.mark.reference
def test_big_obj_matches_reference_live(pkg, ref, tmp_path):
    path = str(tmp_path / "big.obj")
    _write_big_obj(pkg, path)
    ours, _ = _ours(pkg, path, False, **TRANSFORM)
    _same_multiset(ours, _rows(*ref.load_obj(path, **TRANSFORM)))


def test_obj_errors(pkg, tmp_path):
    bad = tmp_path / "bad.obj"
    bad.write_text("v 1 2\nf 1 1 1\n")
    with pytest.raises(pkg.Or3Error):
        pkg.load_obj(str(bad))
    oob = tmp_path / "oob.obj"
    oob.write_text("v 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2 9\n")
    with pytest.raises(pkg.Or3Error):
        pkg.load_obj(str(oob))
    with pytest.raises(pkg.Or3Error):
        pkg.load_obj(str(tmp_path / "missing.obj"))
