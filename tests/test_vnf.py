""".vnf scene files (vmr_load_vnf): the reference's node syntax
(nodes/lex.go, nodes/parser.go) and the PreRender steps that turn nodes into
geometry (polymesh/init.go triangulation, the lights' meshes, the camera).

A scene written by scenes.to_vnf and loaded back must be the scene
scenes.vnf_order describes (the same geoms in the loader's order), bit for
bit: CPU tests compare the host-side accelerators, camera and parse
results on a host-only context; GPU tests compare renders, which must be
identical images.
"""
import numpy as np
import pytest

import vermeer_gb300 as vg
from vermeer_gb300 import scenes

INVALID, UNSUPPORTED = -1, -7


def _same(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return a.shape == b.shape and a.dtype == b.dtype and a.tobytes() == b.tobytes()


def _write(tmp_path, name, text):
    p = tmp_path / name
    p.write_text(text)
    return str(p)


def _load_err(ctx, path):
    with pytest.raises(vg.VmrError) as e:
        ctx.load_vnf(path)
    return e.value.code, str(e.value)


MINI = """# a one-triangle scene
ShaderStd { Name "white" DiffuseColour rgb 1 1 1 DiffuseStrength float 1 }
PolyMesh {
  Name "tri"
  Verts 1 4 point 0 0 0  1 0 0  1 1 0  0 1 0   # a quad
  PolyCount 1 int 4
  FaceIdx 4 int 0 1 2 3
  Shader 1 string "white"
}
Camera { Name "camera" Type "LookAt" From 1 1 point 0 0 -3 To 1 1 point 0 0 0 Roll 1 1 float 0 Up 0 1 0 Fov 40 }
Globals { XRes 32 YRes 16 }
OutputHDR { Filename "out.hdr" }
"""


def test_vnf_minimal_scene(tmp_path):
    host_ctx = vg.Context(-1)  # its own context: geom ids start at 0
    info = host_ctx.load_vnf(_write(tmp_path, "mini.vnf", MINI))
    assert (info["width"], info["height"], info["max_iter"]) == (32, 16, 0)  # a Globals node's own defaults
    assert info["n_geoms"] == 1 and info["n_shaders"] == 1 and info["n_lights"] == 0
    assert info["camera"] == "camera" and info["output_hdr"] == "out.hdr" and info["output_float"] == ""
    # PolyCount 4 fans into (0,1,2), (0,2,3) (polymesh/init.go)
    exp = host_ctx.mesh_export(0)
    assert sorted(map(tuple, np.asarray(exp["idxp"]).reshape(-1, 3).tolist())) == [(0, 1, 2), (0, 2, 3)]
    # LookAt (camera.go:113-190) with Roll 0 and the aspect from Globals
    cam = host_ctx.get_camera()
    ref = scenes.lookat_camera((0, 0, -3), (0, 0, 0), (0, 1, 0), 40.0, 32 / 16)
    assert np.array_equal(cam["m"], ref["m"])
    for k in ("tan_theta_focal", "aspect", "focal"):
        assert cam[k] == ref[k], k
    host_ctx.close()


def test_vnf_one_transform_is_loaded(tmp_path):
    """A PolyMesh Transform of one matrix (rows as written) loads; the
    accelerator stays the object-space one, as PolyMesh builds it."""
    text = MINI.replace('  Shader 1 string "white"\n', '  Shader 1 string "white"\n  Transform 1 matrix '
                        '1 0 0 0.25 0 1 0 0 0 0 1 0 0 0 0 1\n')
    a, b = vg.Context(-1), vg.Context(-1)
    try:
        a.load_vnf(_write(tmp_path, "xf.vnf", text))
        b.load_vnf(_write(tmp_path, "plain.vnf", MINI))
        ea, eb = a.mesh_export(0), b.mesh_export(0)
        for k in ea:
            assert _same(ea[k], eb[k]), k
    finally:
        a.close()
        b.close()


def test_vnf_defaults_without_globals(host_ctx, tmp_path):
    text = MINI.replace("Globals { XRes 32 YRes 16 }", "")
    info = host_ctx.load_vnf(_write(tmp_path, "noglobals.vnf", text))
    assert (info["width"], info["height"], info["max_iter"]) == (1024, 1024, 16)  # core.Init's defaults


@pytest.mark.parametrize("bad,code,what", [
    (MINI.replace("  Shader 1 string \"white\"\n", ""), INVALID, "required field Shader"),
    (MINI.replace("PolyCount", "PolyCnt"), INVALID, "PolyCnt"),
    (MINI.replace("Globals {", "Proc {"), INVALID, "XRes"),
    (MINI + 'Proc { Name "p" Handler "wfobj" Data "a.obj" BMin 1 1 point 0 0 0 BMax 1 1 point 1 1 1 }\n',
     UNSUPPORTED, "wfobj"),
    (MINI + 'GeomInstance { Name "i" Geom "tri" BMin 1 1 point 0 0 0 BMax 1 1 point 1 1 1 '
     'Transform 1 matrix 1 0 0 0 0 1 0 0 0 0 1 0 0 0 0 1 }\n'
     'GeomInstance { Name "j" Geom "i" BMin 1 1 point 0 0 0 BMax 1 1 point 2 2 2 '
     'Transform 1 matrix 1 0 0 0 0 1 0 0 0 0 1 0 0 0 0 1 }\n', UNSUPPORTED, "instances of instances"),
    (MINI + 'GeomInstance { Name "i" Geom "nothing" BMin 1 1 point 0 0 0 BMax 1 1 point 1 1 1 '
     'Transform 1 matrix 1 0 0 0 0 1 0 0 0 0 1 0 0 0 0 1 }\n', INVALID, "unable to find geom nothing"),
    (MINI.replace("rgb 1 1 1", "rgbtex \"wood.tga\""), UNSUPPORTED, "rgbtex"),
    (MINI.replace("\"white\"\n}", "\"black\"\n}"), INVALID, "shader black"),
    (MINI.replace("Name \"camera\"", "Name \"cam2\""), INVALID, "no camera"),
    (MINI.replace("FaceIdx 4 int 0 1 2 3", "FaceIdx 4 int 0 1 2 7"), INVALID, "out of range"),
    (MINI.replace("Verts 1 4 point", "Verts 1 4 vec3"), INVALID, "point"),
    (MINI.replace("Fov 40", "Fov 40 Fov 41"), INVALID, "already"),
    (MINI + "Bogus {\n}\n", INVALID, "unknown node type Bogus"),
])
def test_vnf_errors(host_ctx, tmp_path, bad, code, what):
    c, msg = _load_err(host_ctx, _write(tmp_path, "bad.vnf", bad))
    assert c == code and what in msg, msg
    assert "bad.vnf:" in msg


def test_vnf_error_names_the_line(host_ctx, tmp_path):
    text = MINI.replace("  FaceIdx 4 int 0 1 2 3", "  FaceIdx 4 int 0 1 2 3\n  Colour 1")
    _, msg = _load_err(host_ctx, _write(tmp_path, "line.vnf", text))
    assert "line.vnf:8:" in msg, msg  # line 1 is the comment


SCENES = {
    "small_room": lambda: scenes.small_room(1024, seed=3),
    "disk_thin_lens": lambda: scenes.small_room_disk(1024, seed=4),
    "spheres": lambda: scenes.small_room_spheres(1024, seed=5),
    "motion": lambda: scenes.small_room_motion(1024, seed=6, motion_mode=1),
    "quads_filter": lambda: dict(scenes.small_room_ext(1024, seed=7), pixel_filter={"kind": 1}),
    "transformed": lambda: _transformed(scenes.small_room(1024, seed=8)),
}


def _transformed(sc):
    """The soup with a PolyMesh Transform (a turn about y and a lift)."""
    c, s_ = np.cos(0.3), np.sin(0.3)
    m = np.array([[c, 0, s_, 0], [0, 1, 0, 0.02], [-s_, 0, c, 0], [0, 0, 0, 1]], np.float32)
    meshes = [dict(mm) for mm in sc["meshes"]]
    soup = max(range(len(meshes)), key=lambda g: len(meshes[g].get("idxp", ())))
    meshes[soup]["transform"] = m.T.reshape(16)  # column-major
    return dict(sc, meshes=meshes)


def _host_pair(name, tmp_path, w=40, h=30):
    import vermeer_gb300 as vg_
    sc = SCENES[name]()
    path = _write(tmp_path, name + ".vnf", scenes.to_vnf(sc, w, h))
    motion_fixed = any(m.get("motion_mode", 0) == 1 for m in sc["meshes"])
    return sc, path, motion_fixed, vg_


@pytest.mark.parametrize("name", sorted(SCENES))
def test_vnf_round_trip_builds_the_same_scene(tmp_path, name):
    """Host-only contexts: every accelerator, the top level and the camera
    of the loaded file equal those of the scene built directly."""
    sc, path, mf, vg_ = _host_pair(name, tmp_path)
    a = vg_.Context(-1)
    b = vg_.Context(-1)
    try:
        info = a.load_vnf(path, motion_fixed=mf)
        ref = scenes.vnf_order(sc)
        ids = b.load_scene(ref)
        assert info["n_geoms"] == len(ids)
        for g in range(len(ids)):
            if "sphere" in ref["meshes"][g]:
                continue
            ea, eb = a.mesh_export(g), b.mesh_export(ids[g])
            for k in ea:
                assert _same(ea[k], eb[k]), (g, k)
        sa, sb = a.scene_export(len(ids)), b.scene_export(len(ids))
        for k in sa:
            assert _same(sa[k], sb[k]), k
        ca, cb = a.get_camera(), b.get_camera()
        for k in ca:
            assert _same(ca[k], cb[k]), k
    finally:
        a.close()
        b.close()


# ------------------------------------------------------------------ GPU ----
@pytest.mark.gpu
@pytest.mark.parametrize("name", ["small_room", "disk_thin_lens", "spheres", "motion", "transformed"])
def test_vnf_render_equals_direct_scene(ctx, tmp_path, name):
    sc, path, mf, _ = _host_pair(name, tmp_path)
    ctx.load_scene(scenes.vnf_order(sc))
    ref, _ = ctx.render(40, 30, 0, 3, 5)
    info = ctx.load_vnf(path, motion_fixed=mf)
    got, _ = ctx.render(info["width"], info["height"], 0, 3, 5)
    assert got.tobytes() == ref.tobytes()


@pytest.mark.gpu
def test_vnf_path_render_with_quads_and_filter(ctx, tmp_path):
    sc, path, _, _ = _host_pair("quads_filter", tmp_path)
    ctx.load_scene(scenes.vnf_order(sc))
    ref, _ = ctx.render_path(40, 30, 0, 4, 5, max_depth=4)
    ctx.load_vnf(path)
    got, _ = ctx.render_path(40, 30, 0, 4, 5, max_depth=4)
    assert got.tobytes() == ref.tobytes()
    assert float(got.mean()) > 0.0


# ------------------------------------------- transforms, groups, includes ----
def _write_groups(tmp_path, camera_keys=True):
    sc = scenes.small_room_groups(1024, seed=4, camera_keys=camera_keys)
    extra = {}
    text = scenes.to_vnf(sc, 48, 40, extra_files=extra)
    for name, body in extra.items():
        _write(tmp_path, name, body)
    return sc, _write(tmp_path, "groups.vnf", text), extra


def test_vnf_groups_keys_and_debug_shader_load(tmp_path):
    """GeomInstance, Proc (Handler "vnf", its geoms in the Data file),
    PolyMesh Transform keys, camera LocalToWorld keys and DebugShader load:
    the top level holds every geom but the Proc's children, the camera's
    key 0 is the first matrix, and the Data file is found beside the scene."""
    sc, path, extra = _write_groups(tmp_path)
    assert len(extra) == 1
    c = vg.Context(-1)
    try:
        info = c.load_vnf(path)
        children = {k for m in sc["meshes"] if "proc" in m for k in m["proc"]}
        assert info["n_geoms"] == len(sc["meshes"]) - len(children)
        assert info["n_shaders"] == len(sc["shaders"])
        cam = c.get_camera()
        assert _same(cam["m"], np.asarray(sc["camera"]["keys"][0], np.float32))
    finally:
        c.close()


def test_vnf_include_adds_the_file_in_prerender_order(tmp_path):
    """An Include node (builtin/misc/include.go) parses its file at
    PreRender: its geoms join the scene after the including file's geoms and
    the meshes of the lights before it, its shaders and camera are found by
    name."""
    inc = _write(tmp_path, "part.vnf",
                 'ShaderStd { Name "red" DiffuseColour rgb 1 0 0 DiffuseStrength float 1 }\n'
                 'PolyMesh { Name "t2" Verts 1 3 point 0 0 1  1 0 1  0 1 1 Shader 1 string "red" }\n')
    text = MINI.replace('Shader 1 string "white"', 'Shader 1 string "red"') + 'Include { Filename "part.vnf" }\n'
    c = vg.Context(-1)
    try:
        info = c.load_vnf(_write(tmp_path, "main.vnf", text))
        assert info["n_geoms"] == 2 and info["n_shaders"] == 2
        assert c.mesh_info(1)["n_tris"] == 1  # the included triangle is the second geom
    finally:
        c.close()
    assert inc


GOLDEN_NODES = __import__("os").path.join(__import__("os").path.dirname(__file__), "golden", "quickstart_nodes.vnf")

# What each documented example needs around it to make a scene: the shaders
# it names, a geom for the camera to see, and a camera unless it is one.
_SCENE = ('ShaderStd { Name "mtl2" DiffuseColour rgb 1 1 1 DiffuseStrength float 1 }\n'
          'ShaderStd { Name "lightmtl" EmissionColour rgb 1 1 1 EmissionStrength float 5 '
          'DiffuseColour rgb 0 0 0 DiffuseStrength float 1 }\n'
          'PolyMesh { Name "othergeom" Verts 1 3 point 0 0 0  1 0 0  0 1 0 Shader 1 string "mtl2" }\n')
_CAMERA = 'Camera { Name "camera" Type "LookAt" From 1 1 point 0 0 -3 To 1 1 point 0 0 0 Roll 1 1 float 0 Up 0 1 0 }\n'


def _examples():
    text = open(GOLDEN_NODES).read()
    blocks = [b for b in text.split("# docs/quickstart.rst:") if b.strip()]
    return [(int(b.split("\n", 1)[0]), b.split("\n", 1)[1]) for b in blocks]


def test_vnf_reference_documented_examples(tmp_path):
    """The node examples of the reference's quickstart guide, loaded as
    written (each inside a minimal scene).  Expected outcomes: the guide's
    PolyMesh has no Name, a required field, which the reference's parser
    reports (nodes/parser.go:834-836) and this loader refuses; with a Name it
    loads (two vertex keys, the one-key normals ignored as TraceMotionElems
    ignores them, the identity transform); the ShaderStd and DebugShader
    examples use texture maps (rgbtex), which libvmr does not render;
    "GaussFilter" is not a registered node type (the reference registers
    GaussianFilter); the Proc example uses the wfobj handler; the LookAt
    camera with two From and Roll keys loads as a camera with two motion
    keys; everything else loads."""
    ex = _examples()
    assert len(ex) >= 14
    seen = {}
    for line, body in ex:
        node = body.strip().split()[0]
        seen[node] = line
        scene = _SCENE + body + ("" if node == "Camera" else _CAMERA)
        c = vg.Context(-1)
        try:
            path = _write(tmp_path, f"ex{line}.vnf", scene)
            if node == "PolyMesh":
                code, msg = _load_err(c, path)
                assert code == INVALID and "Name" in msg
                named = scene.replace("PolyMesh {\n", 'PolyMesh {\n  Name "quad"\n', 1)
                info = c.load_vnf(_write(tmp_path, f"ex{line}n.vnf", named))
                assert info["n_geoms"] == 2 and c.mesh_info(1)["n_tris"] == 2
            elif node in ("ShaderStd", "DebugShader"):
                code, msg = _load_err(c, path)
                assert code == UNSUPPORTED and "rgbtex" in msg, msg
            elif node == "GaussFilter":
                code, msg = _load_err(c, path)
                assert code == INVALID and "GaussFilter" in msg
            elif node == "Proc":
                code, msg = _load_err(c, path)
                assert code == UNSUPPORTED and "wfobj" in msg
            else:
                info = c.load_vnf(path)
                if node == "GeomInstance":
                    assert info["n_geoms"] == 2
                if node in ("DiskLight", "SphereLight", "QuadLight", "TriLight"):
                    assert info["n_lights"] == 1
        finally:
            c.close()
    assert {"Globals", "PolyMesh", "ShaderStd", "DebugShader", "Camera", "DiskLight", "SphereLight", "QuadLight",
            "TriLight", "OutputHDR", "OutputFloat", "AiryFilter", "GaussFilter", "Proc", "GeomInstance"} <= set(seen)


def test_vnf_documented_lookat_camera_has_two_keys(orc):
    """The guide's camera: From 2 keys (the same point), To 1 key, Roll 0 and
    0.1.  calcLookatMatrices walks From's keys at times 0 and 1/2 and lerps
    Roll there: 0 and 0.05; the keys differ by that roll only."""
    ex = dict((b.strip().split()[0], b) for _, b in _examples())
    import tempfile
    with tempfile.TemporaryDirectory() as d:
        p = __import__("os").path.join(d, "cam.vnf")
        open(p, "w").write(_SCENE + ex["Camera"])
        c = vg.Context(-1)
        try:
            c.load_vnf(p)
            keys = c.get_camera_keys()
        finally:
            c.close()
    assert keys.shape == (2, 16)
    m0, m1 = keys[0].reshape(4, 4).T, keys[1].reshape(4, 4).T
    assert np.array_equal(m0[:3, 3], np.float32([0, 0.85, 4])) and np.array_equal(m1[:3, 3], m0[:3, 3])
    assert np.allclose(m0[:3, 0], [1, 0, 0], atol=1e-6)  # roll 0 at key 0
    r = np.arctan2(m1[1, 0], m1[0, 0])  # U = cos(r) u + sin(r) v with v = (0, -1, 0)
    assert abs(abs(r) - 0.05) < 1e-6


@pytest.mark.gpu
@pytest.mark.parametrize("camera_keys", [False, True])
def test_vnf_groups_render_as_the_oracle(ctx, orc, tmp_path, camera_keys):
    """The group scene written to .vnf (Proc Data file beside it) and loaded
    by vmr_load_vnf renders the oracle's image of the scene, with the render
    tests' tolerance (the loaded top level orders the geoms as the file does,
    which changes no hit)."""
    sc, path, _ = _write_groups(tmp_path, camera_keys)
    ctx.load_vnf(path)
    got, _ = ctx.render(48, 40, 0, 3, 5)
    ref = orc.Render(sc).run(48, 40, 0, 3, 5)
    ok = np.abs(got - ref) <= 1e-5 * (1.0 + np.abs(ref))
    assert ok.all(-1).mean() >= 0.999 and np.abs(got - ref).mean() <= 1e-6
