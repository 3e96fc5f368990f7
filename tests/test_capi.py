"""The C-ABI library loads and exports every function include/vmr.h declares;
host-only contexts report errors with the documented status codes."""
import ctypes
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for f in os.listdir(os.path.join(ROOT, "include")):
        if f.endswith(".h"):
            src = open(os.path.join(ROOT, "include", f)).read()
            src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
            names |= set(re.findall(r"^\s*(?:int|const char\s*\*|void)\s+(vmr_\w+)\s*\(", src, re.M))
    return sorted(names)


def test_library_exports_every_declared_symbol():
    from vermeer_gb300 import _lib
    L = _lib.load()
    names = declared_functions()
    assert len(names) >= 15
    for n in names:
        assert hasattr(L, n), f"libvmr does not export {n}"
    assert L.vmr_abi_version() == 1


def test_binding_covers_header():
    from vermeer_gb300 import _lib
    assert set(declared_functions()) <= set(_lib.exported_symbols()) | set(_lib.extra_symbols())


def test_host_only_context_refuses_trace(host_ctx):
    import vermeer_gb300 as vg
    from vermeer_gb300 import scenes
    v, ip = scenes.triangle_soup(50, 1)
    g = host_ctx.mesh_build(v, ip)
    with pytest.raises(vg.VmrError) as e:
        host_ctx.trace_mesh(g, scenes.incoherent_rays(10, 1))
    assert e.value.code == -7


def test_upload_validates_reference_nodes(host_ctx, orc):
    """vmr_mesh_upload accepts the oracle-built (reference-layout) tree and
    rejects out-of-range leaf ranges."""
    import vermeer_gb300 as vg
    from vermeer_gb300 import scenes
    v, ip = scenes.triangle_soup(300, 2)
    ex = orc.Mesh(v, ip).export()
    host_ctx.mesh_upload(v, ex["idxp"], ex["accel_idx"], nodes=ex["nodes"], bounds=ex["bounds"])
    bad = ex["accel_idx"].copy()
    bad[0] = 300
    with pytest.raises(vg.VmrError):
        host_ctx.mesh_upload(v, ex["idxp"], bad, nodes=ex["nodes"], bounds=ex["bounds"])


def test_null_context_is_rejected():
    from vermeer_gb300 import _lib
    L = _lib.load()
    assert L.vmr_destroy(None) == -1
    assert L.vmr_sync(None) == -1


@pytest.mark.gpu
def test_contexts_run_concurrently(orc):
    """One context per host thread (the Go wrapper's goroutine rule): two
    threads tracing and path tracing at the same time on their own contexts
    get the results of running alone, bit for bit."""
    import threading

    import vermeer_gb300 as vg
    from vermeer_gb300 import scenes

    v, ip = scenes.triangle_soup(50000, 91, edge=0.01)
    rays = scenes.incoherent_rays(300000, 92)
    room = scenes.small_room_ext(2048, seed=93)

    def work(ctx):
        g = ctx.mesh_build(v, ip)
        hits = ctx.trace_mesh(g, rays)
        ctx.load_scene(room)
        img, _ = ctx.render_path(64, 48, 0, 4, 7, max_depth=4)
        return hits, img

    alone = vg.Context(0)
    try:
        ref_hits, ref_img = work(alone)
    finally:
        alone.close()
    ctxs = [vg.Context(0), vg.Context(0)]
    out = [None, None]
    errs = []

    def run(k):
        try:
            for _ in range(3):
                out[k] = work(ctxs[k])
        except Exception as e:  # reported below
            errs.append(e)

    try:
        th = [threading.Thread(target=run, args=(k,)) for k in range(2)]
        for t in th:
            t.start()
        for t in th:
            t.join()
        assert not errs, errs
        for hits, img in out:
            for key in ("prim", "t", "u", "v", "w"):
                assert np.asarray(hits[key]).tobytes() == np.asarray(ref_hits[key]).tobytes(), key
            assert img.tobytes() == ref_img.tobytes()
    finally:
        for c in ctxs:
            c.close()


@pytest.mark.gpu
def test_bounded_wait_runs_out_and_the_context_stays_usable(orc):
    """The failure path of the kernels' bounded waits, on purpose: a wait on
    an mbarrier that nothing arrives at gives up after its bound, the kernel
    reports through the error word (VMR_ERR_TIMEOUT) and returns; the same
    context then traces and runs the guide network as before."""
    import vermeer_gb300 as vg
    from vermeer_gb300 import scenes

    ctx = vg.Context(0)
    try:
        ms = ctypes.c_float()
        rc = ctx.L.vmr_selftest_wait(ctx.h, ctypes.byref(ms))
        assert rc == -4, rc  # VMR_ERR_TIMEOUT
        assert 1.0 < ms.value < 5000.0, ms.value
        v, ip = scenes.triangle_soup(4096, 94, edge=0.02)
        rays = scenes.incoherent_rays(8192, 95)
        g = ctx.mesh_build(v, ip)
        got = ctx.trace_mesh(g, rays)
        ref = orc.Mesh(v, ip).trace(rays)
        assert np.array_equal(got["prim"], ref["prim"])
        ctx.guide_init(1)
        rng = np.random.default_rng(96)
        pos = rng.random((1000, 3)).astype(np.float32)
        nrm = rng.standard_normal((1000, 3)).astype(np.float32)
        nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
        out = ctx.guide_forward(pos, nrm, nrm, np.zeros(3, np.float32), np.ones(3, np.float32))
        assert np.isfinite(np.asarray(out)).all()
    finally:
        ctx.close()
