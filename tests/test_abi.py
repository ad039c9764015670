"""The C ABI surface, without a GPU: the library loads, exports every entry
point include/vt.h declares, its struct layouts match the Python mirror, and
the host-only calls (generators, camera, argument checks) behave."""
import ctypes as C
import re
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent


def declared_functions():
    src = (ROOT / "include" / "vt.h").read_text()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    names = set(re.findall(r"\b(vt_[a-z0-9_]+)\s*\(", src))
    return sorted(names)


def test_exports_every_declared_symbol(vtlib):
    lib = vtlib.load()
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, f"libvt.so lacks {missing}"
    assert len(declared_functions()) >= 30


def test_python_mirror_covers_header(vtlib):
    assert set(declared_functions()) <= set(vtlib._SIGNATURES), \
        sorted(set(declared_functions()) - set(vtlib._SIGNATURES))


def test_struct_layouts_match_c(vtlib, tmp_path):
    prog = tmp_path / "sizes.c"
    prog.write_text(
        '#include <stdio.h>\n#include <stddef.h>\n#include "vt.h"\n'
        "int main(void){printf(\"%zu %zu %zu %zu %zu %zu %zu %zu %zu\\n\", sizeof(vt_camera), sizeof(vt_params),"
        " sizeof(vt_hit), sizeof(vt_stats), sizeof(vt_gen_desc), sizeof(vt_world_info), sizeof(vt_world_desc),"
        " offsetof(vt_gen_desc, seed), sizeof(vt_tuning));return 0;}\n")
    exe = tmp_path / "sizes"
    subprocess.run(["gcc", "-std=c99", "-I", str(ROOT / "include"), str(prog), "-o", str(exe)], check=True)
    got = [int(v) for v in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()]
    want = [C.sizeof(vtlib.Camera_t), C.sizeof(vtlib.Params_t), vtlib.HIT_DTYPE.itemsize, C.sizeof(vtlib.Stats_t),
            C.sizeof(vtlib.GenDesc_t), C.sizeof(vtlib.WorldInfo_t), C.sizeof(vtlib.WorldDesc_t),
            vtlib.GenDesc_t.seed.offset, C.sizeof(vtlib.Tuning_t)]
    assert got == want


def test_header_is_plain_c99(tmp_path):
    prog = tmp_path / "h.c"
    prog.write_text('#include "vt.h"\nint main(void){return 0;}\n')
    subprocess.run(["gcc", "-std=c99", "-pedantic", "-Werror", "-I", str(ROOT / "include"), str(prog), "-o",
                    str(tmp_path / "h")], check=True)


def test_abi_version_and_status_strings(vtlib):
    lib = vtlib.load()
    assert lib.vt_abi_version() == 1
    assert lib.vt_status_string(0) == b"ok"
    assert lib.vt_status_string(4) == b"device index out of range"


def test_null_arguments_are_rejected(vtlib):
    lib = vtlib.load()
    assert lib.vt_ctx_create(0, None) == 1
    assert lib.vt_ctx_destroy(None) == 1
    assert lib.vt_world_destroy(None) == 1
    assert lib.vt_render(None, None, None, None, None, None) == 1
    assert lib.vt_gen_world(None, None, 0, 1) == 1
    assert lib.vt_world_generate(None, None, None) == 1
    assert lib.vt_world_download_dense(None, None, 0, None) == 1


def test_generator_rejects_bad_sizes(vtlib):
    d = vtlib.gen_desc((16, 16, 16))
    out = np.zeros(10, dtype=np.uint8)
    assert vtlib.load().vt_gen_world(C.byref(d), out.ctypes.data, out.nbytes, 1) == 1


def test_generator_layers_and_water(vtlib):
    d = vtlib.gen_desc((64, 128, 48), seed=7)
    m = vtlib.gen_world(d, threads=3)
    lib = vtlib.load()
    for (x, z) in ((0, 0), (13, 40), (63, 47), (31, 5)):
        h = lib.vt_gen_height(C.byref(d), x, z)
        col = m[z, :, x]
        assert col[h - 1] == 1 and all(col[max(h - 4, 0):h - 1] == 2) and all(col[:max(h - 4, 0)] == 3)
        above = col[h:]
        assert all(above[: max(0, 56 - h)] == 4) and all(above[max(0, 56 - h):] == 0)


def test_generator_threads_do_not_change_bytes(vtlib):
    d = vtlib.gen_desc((96, 80, 64), seed=3, trees=12, caves=True)
    a = vtlib.gen_world(d, threads=1)
    b = vtlib.gen_world(d, threads=5)
    assert np.array_equal(a, b)
    assert (a == 5).sum() > 0 and (a == 6).sum() > 0


def test_camera_look_basis(vtlib):
    cam = vtlib.Camera(pos=(1, 2, 3), yaw=0.0, pitch=0.0, fov=np.pi / 2, width=64, height=32).as_uniform_data()
    v = np.array(cam.view).reshape(4, 4)
    assert np.allclose(v[:3, :3], np.eye(3), atol=1e-7)
    assert cam.tan_half_fov == pytest.approx(1.0, abs=1e-6)
    cam = vtlib.Camera(pos=(0, 0, 0), yaw=0.5, pitch=-0.3, fov=1.2, width=8, height=8).as_uniform_data()
    v = np.array(cam.view).reshape(4, 4)[:3, :3].astype(np.float64)
    assert np.allclose(v @ v.T, np.eye(3), atol=1e-6)
    fwd = v[2]
    assert fwd[1] == pytest.approx(np.sin(-0.3), abs=1e-6)     # negative pitch looks down
    assert cam.tan_half_fov == pytest.approx(np.tan(0.6), rel=1e-6)


def test_camera_rotate_mirrors_reference(vtlib):
    cam = vtlib.Camera()
    cam.rotate(100.0, -50.0)
    assert cam.pitch == pytest.approx(0.1) and cam.yaw == pytest.approx(-0.05)
    cam.rotate(1e6, 0.0)
    assert cam.pitch == pytest.approx(np.pi / 2)


def test_gen_camera_above_terrain(vtlib):
    d = vtlib.gen_desc((128, 128, 128), seed=11)
    lib = vtlib.load()
    for s in range(5):
        cam = vtlib.gen_camera(d, s, 640, 360)
        x, y, z = cam.pos[0], cam.pos[1], cam.pos[2]
        h = lib.vt_gen_height(C.byref(d), int(x), int(z))
        assert y == pytest.approx(max(h, 56.0) + 10.5)
        fwd = np.array(cam.view).reshape(4, 4)[2, :3]
        assert -0.51 <= fwd[1] <= 0.0


def test_no_device_here_is_an_error_not_a_crash(vtlib):
    lib = vtlib.load()
    h = C.c_void_p()
    st = lib.vt_ctx_create(0, C.byref(h))
    if st == 0:
        lib.vt_ctx_destroy(h)
        pytest.skip("a GPU is present")
    assert st == 6


def test_unorm8_table():
    """The device table of float(i) / 255.0f (unorm8.cuh) against the IEEE
    division, entry by entry."""
    import re
    from pathlib import Path
    src = (Path(__file__).resolve().parent.parent / "unnamed-voxel-tracer_gb300" / "csrc" / "unorm8.cuh").read_text()
    body = src[src.index("kUnorm8[256] = {"):src.index("};")]
    vals = [float.fromhex(m) for m in re.findall(r"(0x[0-9a-fp.+-]+)f", body)]
    assert len(vals) == 256
    want = np.arange(256, dtype=np.float32) / np.float32(255)
    assert np.array_equal(np.array(vals, np.float32).view(np.uint32), want.view(np.uint32))
