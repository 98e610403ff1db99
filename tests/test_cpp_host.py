"""The C++ RenderTechnique layer (include/vcr/render_technique.hpp): it
compiles and links against libvcr.so (CPU); on the GPU a C++ driver renders
through TechniquePT / PPM / PPB / NRC, and the PT image equals the same
structs rendered through the C-ABI from Python, bit for bit."""
import ctypes as C
import os
import shutil
import subprocess
import zlib

import numpy as np
import pytest

import vcr
from vcr import _abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "cloudrendering-vulkan_gb300")
SRC = os.path.join(ROOT, "tests", "cpp", "technique_driver.cpp")
RENDERER = os.path.join(ROOT, "tests", "cpp", "renderer_driver.cpp")


def _build(tmp_path, src=SRC):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no g++")
    exe = str(tmp_path / os.path.splitext(os.path.basename(src))[0])
    cmd = [gxx, "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"), src, "-o", exe, "-L", PKG, "-lvcr",
           f"-Wl,-rpath,{PKG}"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
    return exe


def test_cpp_layer_compiles_and_links(tmp_path):
    exe = _build(tmp_path)
    assert os.path.exists(exe)
    syms = subprocess.run(["nm", "-D", "--defined-only", os.path.join(PKG, "libvcr.so")], capture_output=True,
                          text=True).stdout
    for name in ("TechniquePT", "TechniquePPM", "TechniquePPB", "TechniqueNRC", "RenderTechnique6Commit",
                 "Renderer5Apply", "Renderer9LoadCloud", "Renderer12SetTechnique", "RenderTechnique8WriteExr",
                 "RenderTechnique8WritePng"):
        assert name in syms
    assert os.path.exists(_build(tmp_path, RENDERER))


def _read(path):
    raw = open(path, "rb").read()
    off = 0
    out = {}
    for key, typ in (("params", _abi.Params), ("camera", _abi.Camera), ("cloud", _abi.Cloud),
                     ("desc", _abi.GridDesc)):
        n = C.sizeof(typ)
        out[key] = typ.from_buffer_copy(raw[off:off + n])
        off += n
    w, h, passes = np.frombuffer(raw[off:off + 12], np.uint32)
    off += 12
    out["pm_radius"] = float(np.frombuffer(raw[off:off + 4], np.float32)[0])
    off += 4
    out["image"] = np.frombuffer(raw[off:], np.float32).reshape(int(h), int(w), 3)
    out["passes"] = int(passes)
    return out


def _run(exe, mode, out, passes=4):
    res = subprocess.run([exe, mode, str(out), str(passes)], capture_output=True, text=True, timeout=300)
    assert res.returncode == 0, res.stdout + res.stderr
    return res.stdout


@pytest.mark.gpu
def test_technique_pt_equals_the_c_abi_path(cuda, tmp_path):
    exe = _build(tmp_path)
    _run(exe, "pt", tmp_path / "pt.bin", 4)
    d = _read(tmp_path / "pt.bin")
    size = tuple(int(d["desc"].size[i]) for i in range(3))
    fbm = vcr.fbm_desc(seed=3, octaves=4)
    dense = vcr.fbm_fill_host(size, fbm)
    h, w = d["image"].shape[:2]
    with vcr.Context() as ctx:
        ctx.grid_upload(d["desc"], dense)
        ctx.set_cloud(d["cloud"])
        ctx.set_camera(d["camera"])
        ctx.set_params(d["params"])
        ctx.set_frame(w, h)
        for k in range(d["passes"]):
            ctx.pt_pass(seed=17, pass_index=k)
        ctx.synchronize()
        ref = ctx.image_mean()
        shown = ctx.display()
    np.testing.assert_array_equal(d["image"], ref)
    assert (ref > 0.1).any()
    # RenderTechnique::WriteExr / WritePng: the same frame as files
    from test_image_files import read_exr
    _, _, _, exr, _ = read_exr(str(tmp_path / "pt.bin.exr"))
    np.testing.assert_array_equal(exr, ref)
    _, _, _, half, _ = read_exr(str(tmp_path / "pt.bin.half.exr"))
    np.testing.assert_array_equal(half, ref.astype(np.float16).astype(np.float64))
    png = open(tmp_path / "pt.bin.png", "rb").read()
    idat = png[png.index(b"IDAT") + 4:png.index(b"IEND") - 8]
    rows = np.frombuffer(zlib.decompress(idat), np.uint8).reshape(h, 1 + 4 * w)
    np.testing.assert_array_equal(rows[:, 1:].reshape(h, w, 4), shown)


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["ppm", "ppb", "nrc", "nrcpool"])
def test_other_techniques_render(cuda, tmp_path, mode):
    exe = _build(tmp_path)
    _run(exe, mode, tmp_path / f"{mode}.bin", 3)
    d = _read(tmp_path / f"{mode}.bin")
    img = d["image"]
    assert np.isfinite(img).all() and (img >= 0).all() and img.max() > 0
    if mode in ("ppm", "ppb"):
        assert 0 < d["pm_radius"] < 0.02  # the technique shrinks pushConstants.pmRadius


@pytest.mark.gpu
def test_misuse_throws_vcr_errors(cuda, tmp_path):
    exe = _build(tmp_path)
    out = _run(exe, "misuse", tmp_path / "x.bin")
    assert "misuse errors 3" in out


@pytest.mark.gpu
def test_renderer_edit_session(cuda, tmp_path):
    """vcr::Renderer (the reference's main.cpp orchestration): accumulation
    restarts exactly on edits that change the image, fov and pitch clamp like
    SetFOV / SetRotation, techniques switch, the forward vector is
    Rx(pitch) Ry(yaw) (0, 0, 1), and the final frame equals the same structs
    rendered through the C-ABI."""
    exe = _build(tmp_path, RENDERER)
    res = subprocess.run([exe, str(tmp_path / "r.bin")], capture_output=True, text=True, timeout=300)
    assert res.returncode == 0, res.stdout + res.stderr
    assert "renderer checks 12 of 12" in res.stdout, res.stdout
    fwd = np.array([float(v) for v in res.stdout.split("forward ")[1].split()[:3]])
    p, y = np.radians(20.0), np.radians(30.0)
    rx = np.array([[1, 0, 0], [0, np.cos(p), -np.sin(p)], [0, np.sin(p), np.cos(p)]])
    ry = np.array([[np.cos(y), 0, np.sin(y)], [0, 1, 0], [-np.sin(y), 0, np.cos(y)]])
    np.testing.assert_allclose(fwd, rx @ ry @ np.array([0.0, 0.0, 1.0]), atol=1e-6)
    raw = open(tmp_path / "r.bin", "rb").read()
    off, d = 0, {}
    for key, typ in (("params", _abi.Params), ("camera", _abi.Camera), ("cloud", _abi.Cloud),
                     ("desc", _abi.GridDesc)):
        d[key] = typ.from_buffer_copy(raw[off:off + C.sizeof(typ)])
        off += C.sizeof(typ)
    w, h, passes = (int(v) for v in np.frombuffer(raw[off:off + 12], np.uint32))
    img = np.frombuffer(raw[off + 12:], np.float32).reshape(h, w, 3)
    assert passes == 4 and d["cloud"].density_scaling == 16.0
    size = tuple(int(d["desc"].size[i]) for i in range(3))
    dense = vcr.fbm_fill_host(size, vcr.fbm_desc(seed=3, octaves=4))
    with vcr.Context() as ctx:
        ctx.grid_upload(d["desc"], dense)
        ctx.set_cloud(d["cloud"])
        ctx.set_camera(d["camera"])
        ctx.set_params(d["params"])
        ctx.set_frame(w, h)
        for k in range(passes):
            ctx.pt_pass(seed=23, pass_index=k)
        ctx.synchronize()
        ref = ctx.image_mean()
    np.testing.assert_array_equal(img, ref)
