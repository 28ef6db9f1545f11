"""Scene-file ingest (or3_scene_load_file): host code, no GPU.

Pinned against the reference's own SceneFromExternalFile (golden
tests/golden/scene_ref.npz, and live when the reference is built here):
tests/golden/scene/full.scene.in holds every object type (a transformed .obj
mesh with degree rotations, spheres with layered materials and rates, a
sphere light, floors of all six orientations, an infinite floor whose rates
do not match), textures and an IBL.  The reference adds a mesh's triangles
grouped by material; the reader keeps file order, so the mesh's records are
compared as a multiset and every other object in order.  The accept/reject
verdicts of tests/golden/scene/cases.py must match the reference's.
"""
import os
import sys

import numpy as np
import pytest

from conftest import GOLDEN, golden

sys.path.insert(0, os.path.join(GOLDEN, "scene"))
import cases  # noqa: E402
from cases import stage_scene_dir  # noqa: E402


def _records(sd, info):
    """Our scene as the reference harness's records (kind, in BVH, layers, geometry 24, 4 x 10 layer fields)."""
    n = sd.num_objects
    rec = np.zeros((n, 67))

    def layers(r, begin, count):
        r[2] = count
        for j in range(min(count, 4)):
            m = sd.materials[sd.layer_material[begin + j]]
            mt, _tex, em, col, ior, _ph = m
            r[27 + 10 * j:37 + 10 * j] = [mt, *em, *col, ior, sd.layer_rate[begin + j],
                                          info["textures"][sd.layer_material[begin + j]] is not None]

    for verts, nrm, uv, lay, ids in sd.tris:
        for t in range(verts.shape[0]):
            r = rec[ids[t]]
            r[0], r[1] = 0, 1
            r[3:12] = verts[t].reshape(9)
            r[12:21] = nrm[t].reshape(9)
            r[21:27] = uv[t].reshape(6)
            layers(r, lay[t][0], lay[t][1])
    for cx, cy, cz, rad, b, c, flags, i in sd.spheres:
        r = rec[i]
        r[0], r[1] = (2 if flags else 1), 1
        r[3:7] = [cx, cy, cz, rad]
        layers(r, b, c)
    for kind, axis, off, flip, b, c, i in sd.planes:
        r = rec[i]
        r[0], r[1] = 3, 0
        r[3] = off
        layers(r, b, c)
    return rec


def _sorted_rows(x):
    return x[np.lexsort(np.round(x, 9).T[::-1])]


def _compare(ours, ref, n_mesh):
    assert ours.shape == ref.shape, (ours.shape, ref.shape)
    cols = [c for c in range(67) if c != 1]  # the in-BVH flag differs on purpose (every sphere goes in)
    np.testing.assert_allclose(_sorted_rows(ours[:n_mesh][:, cols]), _sorted_rows(ref[:n_mesh][:, cols]),
                               rtol=1e-12, atol=1e-12)
    np.testing.assert_allclose(ours[n_mesh:][:, cols], ref[n_mesh:][:, cols], rtol=1e-12, atol=1e-15)


def _load_full(pkg, tmp_path):
    path = stage_scene_dir(str(tmp_path))
    sd, info = pkg.load_scene_file(path)
    return path, sd, info


def _ibl_sums(orc, sd):
    rgb = orc.decode_rgbe(sd.env_rgbe.reshape(-1, 4))
    return rgb.reshape(-1, 3).sum(axis=0)


def test_scene_file_matches_reference_golden(pkg, orc, tmp_path):
    g = golden("scene_ref.npz")
    _, sd, info = _load_full(pkg, tmp_path)
    ours = _records(sd, info)
    n_mesh = sd.tris[0][0].shape[0] - 12  # the first triangle block: the mesh, then the floors' 12
    _compare(ours, g["records"], n_mesh)
    assert info["meshes"] == 1 and info["space_partitioning"] == "BVH"
    assert info["ibl_path"] == os.path.join(str(tmp_path), "sky.hdr")
    h, w = sd.env_rgbe.shape[:2]
    assert (w, h) == (int(g["ibl"][0]), int(g["ibl"][1]))
    np.testing.assert_allclose(_ibl_sums(orc, sd), g["ibl"][2:5], rtol=1e-9)
    # the reference's out-of-BVH objects: the "Space Partitioning: False" sphere and the infinite floor
    assert list(np.nonzero(g["records"][:, 1] == 0)[0]) == [n_mesh, len(ours) - 1]


def test_scene_file_cases_match_reference_golden(pkg, tmp_path):
    g = golden("scene_ref.npz")
    for name, want in zip(g["case_names"], g["case_objects"]):
        path = cases.write(str(name), str(tmp_path))
        try:
            sd, _ = pkg.load_scene_file(path)
            got = sd.num_objects
        except pkg.Or3Error:
            got = -1
        assert got == want, (name, got, want)


@pytest.mark.reference
def test_scene_file_matches_reference_live(pkg, ref, tmp_path):
    path, sd, info = _load_full(pkg, tmp_path)
    rec, _ = ref.load_scene_file(path)
    _compare(_records(sd, info), rec, sd.tris[0][0].shape[0] - 12)
    for name in sorted(cases.CASES):
        p = cases.write(name, str(tmp_path))
        r = ref.load_scene_file(p)
        try:
            got = pkg.load_scene_file(p)[0].num_objects
        except pkg.Or3Error:
            got = -1
        assert got == (-1 if r is None else r[0].shape[0]), name


def test_scene_file_errors_and_messages(pkg, tmp_path):
    with pytest.raises(pkg.Or3Error) as e:
        pkg.load_scene_file(str(tmp_path / "absent.scene"))
    assert e.value.code == pkg.abi.OR3_ERR_NOT_FOUND
    p = cases.write("missing_mesh", str(tmp_path))
    with pytest.raises(pkg.Or3Error) as e:
        pkg.load_scene_file(p)
    assert e.value.code == pkg.abi.OR3_ERR_NOT_FOUND and "no_such_mesh.obj" in str(e.value)
    p = cases.write("rates_mismatch", str(tmp_path))
    with pytest.raises(pkg.Or3Error) as e:
        pkg.load_scene_file(p)
    assert e.value.code == pkg.abi.OR3_ERR_INVALID_ARGUMENT and "MaterialRates" in str(e.value)
    # an IBL that cannot be read fails loudly (the reference prints and keeps an empty image)
    with open(tmp_path / "noibl.scene", "w") as fh:
        fh.write("Base Dir: %s\nIBL: nothing.hdr\nObjects:\n%s" % (tmp_path, cases._SPHERE))
    with pytest.raises(pkg.Or3Error) as e:
        pkg.load_scene_file(str(tmp_path / "noibl.scene"))
    assert e.value.code == pkg.abi.OR3_ERR_NOT_FOUND
    # an object without a material is rejected (the reference reads past an empty list)
    with open(tmp_path / "nomat.scene", "w") as fh:
        fh.write("Objects:\nSphere {\n  Radius: 1\n}\n")
    with pytest.raises(pkg.Or3Error):
        pkg.load_scene_file(str(tmp_path / "nomat.scene"))


def test_scene_file_layers_and_ids(pkg, tmp_path):
    _, sd, info = _load_full(pkg, tmp_path)
    n_mesh = sd.tris[0][0].shape[0] - 12
    ids = sd.tris[0][4]
    # ids follow the file: mesh triangles, three spheres, floors (two triangles each), the infinite floor
    assert list(ids[:n_mesh]) == list(range(n_mesh))
    assert [s[7] for s in sd.spheres] == [n_mesh, n_mesh + 1, n_mesh + 2]
    assert list(ids[n_mesh:]) == list(range(n_mesh + 3, n_mesh + 15))
    assert sd.planes[0][6] == n_mesh + 15
    s0 = sd.spheres[0]
    assert s0[5] == 2 and sd.layer_rate[s0[4]:s0[4] + 2] == [0.75, 0.25]
    assert sd.spheres[1][6] == pkg.abi.OR3_SPHERE_LIGHT
    # the infinite floor keeps its first material alone, rate 1
    b, c = sd.planes[0][4], sd.planes[0][5]
    assert c == 1 and sd.layer_rate[b] == 1.0 and sd.materials[sd.layer_material[b]][0] == pkg.abi.OR3_LAMBERT
    tex = [t for t in info["textures"] if t]
    assert tex and all(t == os.path.join(str(tmp_path), "sky.hdr") for t in tex)


def test_loaded_scene_converts_to_a_descriptor(pkg, tmp_path):
    _, sd, _ = _load_full(pkg, tmp_path)
    d, keep = sd.to_c()
    assert d.num_triangles == sd.tris[0][0].shape[0] and d.num_spheres == 3 and d.num_planes == 1
    assert d.env_width > 0 and d.env_rgbe


@pytest.mark.reference
def test_oracle_agrees_with_reference_on_the_scene_file_scene(pkg, orc, ref, tmp_path):
    """The oracle's closest hits on the loaded scene equal the reference's (FP64 both)."""
    _, sd, _ = _load_full(pkg, tmp_path)
    rng = np.random.default_rng(5)
    n = 4000
    o = rng.uniform(-12, 12, (n, 3)) + np.array([0.0, 4.0, 0.0])
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    ids_o, t_o, _ = orc.scene(sd, use_bvh=False).closest(o, d)
    ids_r, t_r, _ = ref.scene(sd, use_bvh=False).closest(o, d)
    assert (ids_o == ids_r).mean() >= 0.999 and (ids_o >= 0).sum() > n // 4
    same = ids_o == ids_r
    np.testing.assert_allclose(t_o[same & (ids_o >= 0)], t_r[same & (ids_o >= 0)], rtol=1e-12)


def test_scene_file_mutations_never_crash(pkg, tmp_path):
    """Seeded mutations of the full scene (lines dropped, repeated or cut, delimiters
    planted) load or fail with a status; the reader never crashes or hangs."""
    path = stage_scene_dir(str(tmp_path))
    text = open(path).read()
    lines = text.split("\n")
    rng = np.random.default_rng(17)
    outcomes = {"ok": 0, "error": 0}
    for k in range(300):
        ls = list(lines)
        for _ in range(int(rng.integers(1, 4))):
            j = int(rng.integers(0, len(ls)))
            op = int(rng.integers(0, 5))
            if op == 0:
                del ls[j]
            elif op == 1:
                ls.insert(j, ls[j])
            elif op == 2:
                ls[j] = ls[j][:int(rng.integers(0, len(ls[j]) + 1))]
            elif op == 3 and ls[j]:
                c = int(rng.integers(0, len(ls[j])))
                ls[j] = ls[j][:c] + "{}:,#"[int(rng.integers(0, 5))] + ls[j][c + 1:]
            else:
                ls.insert(j, "")
        p = tmp_path / ("m%03d.scene" % k)
        p.write_text("\n".join(ls))
        try:
            sd, _ = pkg.load_scene_file(str(p))
            assert sd.num_objects >= 0
            outcomes["ok"] += 1
        except pkg.Or3Error as e:
            assert e.code in (pkg.abi.OR3_ERR_INVALID_ARGUMENT, pkg.abi.OR3_ERR_NOT_FOUND)
            outcomes["error"] += 1
    assert outcomes["ok"] > 0 and outcomes["error"] > 0, outcomes
