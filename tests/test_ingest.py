"""Scene ingestion (hrt_scene_load: PLY, OBJ, Helios XML) against the reference loaders' rules
(core/src/Context_fileIO.cpp) and the reference's OBJ tests (core/tests/Test_OBJ.h), on small
files written here.  Host code of the library only: no GPU."""
import math
import struct

import numpy as np
import pytest

from helios_gb300 import _hrt
from helios_gb300.radiation import Context, HeliosRuntimeError


def verts(T):
    """Triangle vertices from transforms of the canonical triangle (0,0,0), (0,1,0), (1,1,0)."""
    T = np.asarray(T, np.float64).reshape(-1, 4, 4)
    v0 = T[:, :3, 3]
    v1 = v0 + T[:, :3, 1]
    v2 = v1 + T[:, :3, 0]
    return np.stack([v0, v1, v2], axis=1)


def rotate_point(p, theta, phi):
    """core/src/global.cpp:156-204 in FP32: Rz(phi) Ry(theta) p."""
    if theta == 0 and phi == 0:
        return np.asarray(p, np.float32)
    f = np.float32
    st, ct, sp, cp = f(math.sin(f(theta))), f(math.cos(f(theta))), f(math.sin(f(phi))), f(math.cos(f(phi)))
    Ry = np.array([[ct, 0, st], [0, 1, 0], [-st, 0, ct]], np.float32)
    Rz = np.array([[cp, -sp, 0], [sp, cp, 0], [0, 0, 1]], np.float32)
    return (Rz @ Ry) @ np.asarray(p, np.float32)


def write(tmp_path, name, text):
    p = tmp_path / name
    p.write_text(text)
    return str(p)


def test_obj_simple_triangle(hrt_lib, tmp_path):
    """Test_OBJ.h:13-39: one triangle (0,0,0), (1,0,0), (0.5,1,0)."""
    p = write(tmp_path, "tri.obj", "v 0 0 0\nv 1 0 0\nv 0.5 1 0\nf 1 2 3\n")
    f = _hrt.load_scene_file(p)
    assert f["T"].shape == (1, 16) and f["type"].tolist() == [1]
    assert np.allclose(verts(f["T"])[0], [[0, 0, 0], [1, 0, 0], [0.5, 1, 0]], atol=1e-6)


def test_obj_cube_with_materials(hrt_lib, tmp_path):
    """Test_OBJ.h:41-59: a 2 m cube of quads gives 12 triangles of total area 24; triangles are
    grouped by material name and take the material's Kd colour."""
    write(tmp_path, "cube.mtl", "newmtl red\nKd 1 0 0\nnewmtl green\nKd 0 1 0\n")
    vs = [(x, y, z) for x in (-1, 1) for y in (-1, 1) for z in (-1, 1)]
    idx = {v: i + 1 for i, v in enumerate(vs)}
    quads = [[(-1, -1, -1), (-1, 1, -1), (-1, 1, 1), (-1, -1, 1)], [(1, -1, -1), (1, -1, 1), (1, 1, 1), (1, 1, -1)],
             [(-1, -1, -1), (-1, -1, 1), (1, -1, 1), (1, -1, -1)], [(-1, 1, -1), (1, 1, -1), (1, 1, 1), (-1, 1, 1)],
             [(-1, -1, -1), (1, -1, -1), (1, 1, -1), (-1, 1, -1)], [(-1, -1, 1), (-1, 1, 1), (1, 1, 1), (1, -1, 1)]]
    lines = ["mtllib cube.mtl"] + [f"v {x} {y} {z}" for x, y, z in vs]
    for k, q in enumerate(quads):
        lines.append("usemtl " + ("red" if k % 2 else "green"))
        lines.append("f " + " ".join(f"{idx[v]}/1/1" for v in q))
    p = write(tmp_path, "cube.obj", "\n".join(lines) + "\n")
    f = _hrt.load_scene_file(p)
    V = verts(f["T"])
    area = 0.5 * np.linalg.norm(np.cross(V[:, 1] - V[:, 0], V[:, 2] - V[:, 0]), axis=1)
    assert len(f["type"]) == 12 and abs(area.sum() - 24.0) < 1e-4
    # std::map order: "green" faces first, then "red"
    assert np.allclose(f["color"][:6], [0, 1, 0]) and np.allclose(f["color"][6:], [1, 0, 0])


def test_obj_transformations(hrt_lib, tmp_path):
    """Test_OBJ.h:83-108 and loadOBJ's rules: a flat model is scaled by the height itself,
    then rotated (elevation, azimuth) and moved to the origin; YUP turns y up into z."""
    p = write(tmp_path, "tri.obj", "v 0 0 0\nv 1 0 0\nv 0.5 1 0\nf 1 2 3\n")
    origin, height, rot = (5.0, 10.0, 2.0), 3.0, (math.pi / 4, math.pi / 6)
    f = _hrt.load_scene_file(p, origin, height, rot, "ZUP", (1.0, 0.0, 0.0))
    exp = [np.float32(origin) + rotate_point(v, *rot) * np.float32(height)
           for v in ([0, 0, 0], [1, 0, 0], [0.5, 1, 0])]
    assert np.allclose(verts(f["T"])[0], exp, atol=1e-5)
    assert np.allclose(f["color"][0], [1, 0, 0])
    g = _hrt.load_scene_file(p, up_axis="YUP")
    assert np.allclose(verts(g["T"])[0], [[0, 0, 0], [1, 0, 0], [0.5, 0, 1]], atol=1e-6)


def test_obj_errors_and_empty(hrt_lib, tmp_path):
    """Test_OBJ.h:205-240: an empty file loads nothing; a missing file, an out-of-range face
    and a wrong extension are errors."""
    assert _hrt.load_scene_file(write(tmp_path, "e.obj", "# nothing\n"))["T"].shape == (0, 16)
    with pytest.raises(_hrt.HrtError, match="could not open"):
        _hrt.load_scene_file(str(tmp_path / "missing.obj"))
    with pytest.raises(_hrt.HrtError, match="out of range"):
        _hrt.load_scene_file(write(tmp_path, "bad.obj", "v 0 0 0\nv 1 0 0\nf 1 2 7\n"))
    with pytest.raises(_hrt.HrtError, match="not PLY, OBJ or XML"):
        _hrt.load_scene_file(write(tmp_path, "tri.txt", "v 0 0 0\n"))


PLY_V = [(0.0, 0.0, 0.0), (1.0, 0.0, 0.0), (1.0, 1.0, 0.0), (0.0, 1.0, 0.0), (0.0, 0.0, 2.0), (1.0, 0.0, 2.0)]
PLY_F = [[0, 1, 2, 3], [0, 1, 5, 4], [0, 0, 1]]  # a quad, a standing quad, a degenerate triangle
PLY_C = [(255, 0, 0), (0, 255, 0), (0, 0, 255), (255, 255, 255), (10, 20, 30), (40, 50, 60)]


def _ply_ascii(tmp_path):
    head = ["ply", "format ascii 1.0", "comment test", f"element vertex {len(PLY_V)}", "property float x",
            "property float y", "property float z", "property uchar red", "property uchar green", "property uchar blue",
            f"element face {len(PLY_F)}", "property list uchar int vertex_indices", "end_header"]
    body = [f"{x} {y} {z} {r} {g} {b}" for (x, y, z), (r, g, b) in zip(PLY_V, PLY_C)]
    body += [" ".join(map(str, [len(fc)] + fc)) for fc in PLY_F]
    return write(tmp_path, "m.ply", "\n".join(head + body) + "\n")


def _ply_binary(tmp_path):
    head = ["ply", "format binary_little_endian 1.0", f"element vertex {len(PLY_V)}", "property float x",
            "property float y", "property float z", "property uchar red", "property uchar green", "property uchar blue",
            f"element face {len(PLY_F)}", "property list uchar int vertex_indices", "end_header"]
    data = b"".join(struct.pack("<fffBBB", *v, *c) for v, c in zip(PLY_V, PLY_C))
    data += b"".join(struct.pack("<B" + "i" * len(fc), len(fc), *fc) for fc in PLY_F)
    p = tmp_path / "b.ply"
    p.write_bytes(("\n".join(head) + "\n").encode() + data)
    return str(p)


def test_ply_ascii_and_binary(hrt_lib, tmp_path):
    """loadPLY (Context_fileIO.cpp:3633-3908): YUP by default (file y is up), polygons
    fan-triangulated from their first vertex, degenerate triangles dropped, colours of the
    first vertex of the face; binary little-endian gives the same arrays."""
    a = _hrt.load_scene_file(_ply_ascii(tmp_path), up_axis="YUP")
    b = _hrt.load_scene_file(_ply_binary(tmp_path), up_axis="YUP")
    assert len(a["type"]) == 4
    for k in ("T", "type", "twosided", "color"):
        assert np.array_equal(a[k], b[k])
    # YUP: Helios (x, y, z) = file (z, x, y), then the base moved to z = 0
    rem = [(z, x, y) for x, y, z in PLY_V]
    zmin = min(v[2] for v in rem)
    rem = [(x, y, z - zmin) for x, y, z in rem]
    exp = [[rem[0], rem[1], rem[2]], [rem[0], rem[2], rem[3]], [rem[0], rem[1], rem[5]], [rem[0], rem[5], rem[4]]]
    assert np.allclose(verts(a["T"]), exp, atol=1e-6)
    assert np.allclose(a["color"][0], np.array(PLY_C[0]) / 255.0)
    h = _hrt.load_scene_file(_ply_ascii(tmp_path), height=2.0, up_axis="ZUP")
    assert np.isclose(verts(h["T"])[:, :, 2].max(), 2.0, atol=1e-6)


def test_xml_primitives_and_data(hrt_lib, tmp_path):
    """loadXML: patches, triangles (from <vertices>), voxels and disks in that order, their
    transforms, and scalar primitive data with twosided_flag."""
    T = " ".join(map(str, [2, 0, 0, 1, 0, 3, 0, 2, 0, 0, 1, 3, 0, 0, 0, 1]))
    xml = f"""<?xml version="1.0"?>
<helios>
  <!-- a comment -->
  <disk><transform>{T}</transform></disk>
  <triangle><vertices>0 0 0 1 0 0 0 1 0</vertices><data_float label="reflectivity_SW">0.25</data_float></triangle>
  <patch><transform>{T}</transform><data_uint label="twosided_flag">0</data_uint><data_double label="temperature">301.5</data_double></patch>
  <voxel><transform>{T}</transform></voxel>
</helios>
"""
    f = _hrt.load_scene_file(write(tmp_path, "s.xml", xml))
    assert f["type"].tolist() == [0, 1, 4, 2]
    assert np.allclose(f["T"][0], [float(x) for x in T.split()])
    assert f["twosided"].tolist() == [0, 1, 1, 1]
    assert np.allclose(verts(f["T"][1])[0], [[0, 0, 0], [1, 0, 0], [0, 1, 0]], atol=1e-6)
    assert f["data"]["temperature"][0] == 301.5 and np.isnan(f["data"]["temperature"][1])
    assert f["data"]["reflectivity_SW"][1] == 0.25
    with pytest.raises(_hrt.HrtError, match="16 values"):
        _hrt.load_scene_file(write(tmp_path, "bad.xml", "<helios><patch><transform>1 2 3</transform></patch></helios>"))
    with pytest.raises(_hrt.HrtError, match="helios"):
        _hrt.load_scene_file(write(tmp_path, "bad2.xml", "<scene></scene>"))


def test_context_loaders(hrt_lib, tmp_path):
    """The Context mirror adds loaded primitives with their areas and primitive data."""
    ctx = Context()
    u = ctx.loadPLY(_ply_ascii(tmp_path))
    assert len(u) == 4 and ctx.getPrimitiveCount() == 4
    assert np.isclose(ctx.getPrimitiveArea(int(u[0])), 0.5)
    v = ctx.loadXML(write(tmp_path, "t.xml", "<helios><triangle><vertices>0 0 0 2 0 0 0 2 0</vertices>"
                                               "<data_float label=\"temperature\">290</data_float></triangle></helios>"))
    assert np.isclose(ctx.getPrimitiveArea(int(v[0])), 2.0)
    assert ctx.getPrimitiveData(int(v[0]), "temperature") == 290.0
    with pytest.raises(HeliosRuntimeError):
        ctx.loadOBJ(str(tmp_path / "m.ply"))
