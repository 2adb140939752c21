"""The C++ drop-in (skity_gb300/adapter: skity::cuda::CUDACanvas, a
skity::Canvas over the C ABI) compiled against the reference's own headers
and software library, with the C ABI replaced by a recorder
(tests/adapter_driver.cc): Skity's Canvas / Path / Paint / Shader /
MaskFilter calls must reach skity_cuda_* with the reference's storage and
values.  CPU only; runs where the reference checkout and its build exist."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = os.environ.get("SKITY_REFERENCE", "/root/reference")
# set_matrix arguments as the driver's stub prints them (%a)
T21 = "0x1p+0 0x0p+0 0x1p+1 0x0p+0 0x1p+0 0x1p+0 0x0p+0 0x0p+0 0x1p+0"
IDENTITY = "0x1p+0 0x0p+0 0x0p+0 0x0p+0 0x1p+0 0x0p+0 0x0p+0 0x0p+0 0x1p+0"


@pytest.fixture(scope="module")
def driver_output(oracle_lib, tmp_path_factory):
    if not os.path.isdir(REF):
        pytest.skip("reference checkout not present")
    oracle_lib.build_reference()
    lib = os.path.join(ROOT, "oracle", "_ref", "libskity_ref_sw.a")
    exe = str(tmp_path_factory.mktemp("adapter") / "adapter_driver")
    cmd = ["g++", "-std=c++17", "-O1", "-DSKITY_CPU", "-DSKITY_RELEASE", "-w",
           "-I" + os.path.join(ROOT, "oracle", "ref", "glm_shim"), "-I" + REF + "/include",
           "-I" + REF, "-I" + REF + "/src", os.path.join(ROOT, "tests", "adapter_driver.cc"),
           os.path.join(ROOT, "skity_gb300", "adapter", "cuda_canvas.cc"), lib, "-lpthread",
           "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([exe], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stderr
    return r.stdout.splitlines()


def test_factory_semantics_match_make_software_canvas(driver_output):
    assert driver_output[0] == "null=1" and driver_output[1] == "empty=1"
    assert driver_output[2] == "create ctx=0x20 w=40 h=30 pixels=1 row_bytes=160"


def test_clear_and_path_storage(driver_output):
    # Canvas::Clear -> DrawPaint(kSrc) -> skity_cuda_canvas_clear, Color4f of ARGB(255,255,128,0)
    assert driver_output[3] == "clear 1 0.501961 0 1"
    d = driver_output[4]
    assert "verbs=0,1,2,3,4,5," in d and "weights=0.5," in d
    assert "points=" + ",".join(str(v) for v in range(1, 19)) + "," in d
    assert "fill_type=1 style=2 cap=1 join=2 blend=3 width=3 miter=5" in d
    assert "fill=0,1,0,0.5 stroke=0,1,0,0.5" in d and d.endswith("blur=0,0")


def test_shaders_and_mask_filter(driver_output):
    lin = driver_output[6]
    assert "shader=1 tile=2 stops=3 offsets=1 p0=0,0 p1=40,30" in lin
    assert "colors=1,0,0,1,0,1,0,0.5,0,0,1,1," in lin and "pos=0,0.25,1," in lin
    assert lin.endswith("blur=1,4.5")
    rad = driver_output[8]
    assert "shader=2 tile=0 stops=3 offsets=0 p0=20,15" in rad and "r=12" in rad


def test_matrix_forwarded_perspective_refused(driver_output):
    # Canvas::Save reaches the C ABI (its save level keeps the path clips);
    # Translate(5, 0) then Translate(0.5, -2): the canvas matrix (a
    # translation of (5.5, -2)) set around the draw; a perspective matrix is
    # outside the GPU path (-5)
    assert driver_output[9:12] == ["save", "save", "set_matrix 0x1p+0 0x0p+0 0x1.6p+2 0x0p+0 "
                                   "0x1p+0 -0x1p+1 0x0p+0 0x0p+0 0x1p+0"]
    assert driver_output[12].startswith("draw verbs=0,1,2,3,4,5,")
    assert driver_output[13:16] == ["restore", "status=0", "status=-5"]
    assert driver_output[16] == "restore"


def test_clip_rect_forwarded(driver_output):
    # Translate(2, 1); ClipRect(1.5, 0, 30, 20) -> device (3.5, 1, 32, 21);
    # ClipRect(-5, 2, 25, 40) -> (-3, 3, 27, 41); the global clip bounds are
    # their intersection (3.5, 3, 27, 21), set before the translation
    assert driver_output[17:21] == ["save", "save", "clip 3.5 3 27 21", "set_matrix 0x1p+0 0x0p+0 0x1p+1 0x0p+0 0x1p+0 0x1p+0 0x0p+0 0x0p+0 0x1p+0"]
    assert driver_output[21].startswith("draw verbs=0,1,2,3,4,5,")
    assert driver_output[22:24] == ["restore", "status=0"]


def test_difference_clip_rect_is_a_path_clip(driver_output):
    # ClipRect(0, 0, 10, 10, kDifference) under Translate(2, 1): the rect's
    # path (Canvas::OnClipRect) clipped on the C ABI canvas at this save
    # level, with the global clip bounds and the canvas matrix of the call
    # (set for the call, then the identity again)
    assert driver_output[24:27] == ["save", "clip 3.5 3 27 21", "set_matrix " + T21]
    assert driver_output[27] == "clip_path op=0 fill=0 verbs=0,1,1,1,5, points=0,0,10,0,10,10,0,10,"
    assert driver_output[28] == "set_matrix " + IDENTITY
    # the draw under it is taken (the path clip is recorded on the state)
    assert driver_output[29:32] == ["save", "clip 3.5 3 27 21", "set_matrix 0x1p+0 0x0p+0 0x1p+1 0x0p+0 0x1p+0 0x1p+0 0x0p+0 0x0p+0 0x1p+0"]
    assert driver_output[32].startswith("draw verbs=0,1,2,3,4,5,")
    assert driver_output[33:37] == ["restore", "status=0", "restore", "restore"]
    # after the Restores the canvas is unclipped and untranslated again
    assert driver_output[37].startswith("draw verbs=0,1,2,3,4,5,")
    assert driver_output[38] == "status=0"


def test_sweep_and_conical_shaders_forwarded(driver_output):
    # MakeSweep(20, 15, 90, 270): GradientInfo radius = (bias, scale) =
    # (-0.25, 2); MakeTwoPointConical keeps both circles
    sweep, conical = driver_output[39], driver_output[40]
    assert "shader=3 tile=1 stops=3 offsets=1 p0=20,15" in sweep and "r=-0.25" in sweep
    assert "shader=4 tile=0 stops=3 offsets=0 p0=5,6 p1=30,20 r=2" in conical
    assert driver_output[41] == "status=0"


def test_color_filters_forwarded(driver_output):
    blend, matrix, gamma = driver_output[42:45]
    assert " filter=1 mode=14 color=80102030 " in blend
    assert " filter=2 mode=0 color=00000000 m=0,1,0,0,0.25,1,0,0,0,0,0,0,1,0,0,0,0,0,0.5,0," in matrix
    assert " filter=4 " in gamma
    assert driver_output[45:48] == ["status=0", "flush", "status=0"]


def test_save_layer_forwarded(driver_output):
    # Save; Translate(3, 2); SaveLayer((1, 1, 21, 11), alpha 0.25, kMultiply):
    # the global clip bounds narrowed to the mapped bounds (4, 3, 24, 13)
    i = driver_output.index("save_layer 1 1 21 11 alpha=0.25 blend=24")
    assert driver_output[i - 4:i] == ["save", "save", "clip 4 3 24 13", "translate 3 2"]
    assert driver_output[i + 1:i + 3] == ["translate -3 -2", "status=0"]
    # the draw inside carries its clip and matrix; Restore of the layer
    # level pops both C-ABI levels, then the outer Save's
    assert driver_output[i + 3:i + 6] == ["save", "clip 4 3 24 13", "set_matrix 0x1p+0 0x0p+0 "
                                          "0x1.8p+1 0x0p+0 0x1p+0 0x1p+1 0x0p+0 0x0p+0 0x1p+0"]
    assert driver_output[i + 6].startswith("draw verbs=0,1,2,3,4,5,")
    assert driver_output[i + 7:i + 11] == ["restore", "restore", "restore", "restore"]


def test_draw_image_rect_forwarded(driver_output):
    line = [l for l in driver_output if l.startswith("image ")]
    assert line == ["image 4x3 alpha_type=2 src=0,0,4,3 dst=5,6,13,12 filter=1 alpha=0.5 blend=3"]
    i = driver_output.index(line[0])
    assert driver_output[i + 1] == "status=0"
    # MakeCUDACanvas(Bitmap*): a canvas over the process-wide context
    assert driver_output[i + 2] == "create ctx=0x30 w=40 h=30 pixels=1 row_bytes=160"
    assert driver_output[i + 3:i + 5] == ["default_ctx=1", "destroy 0x10"]
    assert driver_output[-1] == "destroy 0x10"


def test_scale_rotate_skew_forwarded(driver_output):
    # Translate(3, 2) * Scale(2, 0.5): a radial shader under scale and
    # translation is taken
    i = driver_output.index("default_ctx=1") + 2
    assert driver_output[i:i + 3] == ["save", "save", "set_matrix 0x1p+1 0x0p+0 0x1.8p+1 0x0p+0 "
                                      "0x1p-1 0x1p+1 0x0p+0 0x0p+0 0x1p+0"]
    assert "shader=2" in driver_output[i + 3]
    assert driver_output[i + 4:i + 6] == ["restore", "status=0"]
    # then Rotate(30, 4, 5) and Skew(0.25, 0): the matrix reaching the C ABI
    # is the reference canvas's own GetTotalMatrix, bit for bit
    total = driver_output[i + 6]
    assert total.startswith("total ")
    assert driver_output[i + 7:i + 9] == ["save", "set_matrix " + total[6:]]
    assert driver_output[i + 9].startswith("draw ") and driver_output[i + 10:i + 12] == \
        ["restore", "status=0"]
    # a gradient under the rotation is refused; a ClipRect under it is a
    # path clip of the rect under the rotation (the global clip bounds
    # narrowed by the rotated rect's bounds first), and a draw under it is
    # taken
    assert driver_output[i + 12:i + 16] == ["save", "set_matrix " + total[6:], "restore",
                                            "status=-5"]
    clip = "clip 3.40192 1.33494 26.3923 8.79006"
    assert driver_output[i + 16:i + 21] == [
        clip, "set_matrix " + total[6:],
        "clip_path op=1 fill=0 verbs=0,1,1,1,5, points=0,0,10,0,10,10,0,10,",
        "set_matrix " + IDENTITY, "status=0"]
    assert driver_output[i + 21:i + 24] == ["save", clip, "set_matrix " + total[6:]]
    assert driver_output[i + 24].startswith("draw ")
    assert driver_output[i + 25:i + 28] == ["restore", "status=0", "restore"]


def test_capi_binding_compiles(tmp_path):
    """The module/capi binding of INTEGRATION.md (a skity_canvas handle over
    the CUDA canvas) compiles against the reference's C API headers."""
    if not os.path.isdir(os.path.join(REF, "module", "capi")):
        pytest.skip("reference checkout not present")
    cmd = ["g++", "-std=c++17", "-c", "-w", "-DSKITY_CPU", "-I" + ROOT,
           "-I" + os.path.join(ROOT, "oracle", "ref", "glm_shim"), "-I" + REF + "/include",
           "-I" + REF, "-I" + REF + "/src", "-I" + REF + "/module/capi/include",
           "-I" + REF + "/module/capi/src", os.path.join(ROOT, "tests", "capi_binding.cc"),
           "-o", str(tmp_path / "capi_binding.o")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
