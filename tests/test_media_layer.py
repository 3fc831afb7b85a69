"""Layered-media discretisation (equivalent-medium methods "loc", "har",
"ari") against the reference's own media_layer2model_el_iso and
media_layer2model_el_vti: the oracle bit for bit (CPU), the device within
float rounding (GPU), the drop-in adapter inside the reference's process."""

import os
import sys

import numpy as np
import pytest

from helpers import ref_tree

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
FIX = os.path.join(REPO, "tests", "golden", "media", "layer_el_iso.npz")
FIX_VTI = os.path.join(REPO, "tests", "golden", "media", "layer_el_vti.npz")
FIX_ONE = os.path.join(REPO, "tests", "golden", "media", "layer_onecmp.npz")
FIX_BIN = os.path.join(REPO, "tests", "golden", "media", "bin_model.npz")
VTI_OUT = ("c11", "c33", "c55", "c66", "c13", "rho")
VTI_CASES = [("elastic_vti_prem", "loc"), ("elastic_vti_prem", "ari"),
             ("elastic_vti_thomsen", "loc"), ("elastic_vti_thomsen", "har"),
             ("elastic_vti_thomsen", "ari"),
             ("elastic_vti_cij", "loc"), ("elastic_vti_cij", "har")]


def _fixture():
    from cgfd3d_gb300 import media
    z = np.load(FIX)
    return z, media.read_md3lay(bytes(z["md3lay"]).decode())


def _vti(kind):
    from cgfd3d_gb300 import media
    z = np.load(FIX_VTI)
    return z, media.read_md3lay(bytes(z[kind + "_md3lay"]).decode())


def test_md3lay_parser():
    z, m = _fixture()
    assert m["NI"] == 4 and m["rec"].shape == (4, m["NY"], m["NX"], 10)
    assert np.all(m["rec"][2, :, :, 0] == -800.0)       # the flat interface


METHODS = [("loc", ""), ("har", "_har"), ("ari", "_ari")]


@pytest.mark.parametrize("method,sfx", METHODS)
def test_oracle_matches_reference_bitwise(method, sfx):
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle
    z, m = _fixture()
    got = oracle.layer_el_iso(m, z["x3d"], z["y3d"], z["z3d"], method)
    for g, n in zip(got, ("lam", "mu", "rho")):
        np.testing.assert_array_equal(g.view(np.int32), z[n + sfx].view(np.int32))
    # points on the flat interface take the mean of the two layers
    on = np.isclose(z["z3d"], -800.0)
    assert on.sum() > 100
    if method != "loc":
        # the averaged points are those whose cells straddle an interface
        changed = z["lam" + sfx] != z["lam"]
        assert 500 < changed.sum() < 0.3 * changed.size


@pytest.mark.parametrize("kind,method", VTI_CASES)
def test_oracle_vti_matches_reference_bitwise(kind, method):
    """Bit for bit, including the elastic_vti_cij branch's evaluation of the
    layer above an interface point with the point's own dz (a restatement
    that recomputes dz there differs at 264 points of the loc case)."""
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle
    z, m = _vti(kind)
    assert m["media_type"] == kind and m["rec"].shape[-1] == 19
    got = oracle.layer(m, z["x3d"], z["y3d"], z["z3d"], method)
    for g, n in zip(got, VTI_OUT):
        np.testing.assert_array_equal(g.view(np.int32), z["%s_%s_%s" % (kind, method, n)]
                                      .view(np.int32))


def _one():
    from cgfd3d_gb300 import media
    z = np.load(FIX_ONE)
    g = np.load(FIX)
    return z, g, media.read_md3lay(bytes(z["md3lay"]).decode())


@pytest.mark.parametrize("method", ["loc", "har", "ari"])
def test_oracle_onecmp_matches_reference_bitwise(method):
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle
    z, g, m = _one()
    assert m["media_type"] == "one_component" and m["rec"].shape[-1] == 4
    got = oracle.layer(m, g["x3d"], g["y3d"], g["z3d"], method)[0]
    np.testing.assert_array_equal(got.view(np.int32), z["var_" + method].view(np.int32))


@pytest.mark.parametrize("vis", [False, True])
def test_oracle_bin_matches_reference_bitwise(vis):
    """Binary-volume models (media_bin2model_el_iso / _vis_iso): stored z
    fastest, z decreasing, cropped in x and y, grid points below the model."""
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle
    z = np.load(FIX_BIN)
    g = np.load(FIX)
    got = oracle.bin_model(z, g["x3d"], g["y3d"], g["z3d"], vis)
    for a, k in zip(got, ("Qp", "Qs") if vis else ("rho", "lam", "mu")):
        np.testing.assert_array_equal(a.view(np.int32), z[k].view(np.int32))
    # the grid reaches below the model: those points take its last level
    assert g["z3d"].min() < float(z["origin"][0] + z["spacing"][0] * (z["size"][0] - 1))


def test_pow_guard():
    """cgfd_media_layer_pow_ok (host logic, no device work): the fixtures'
    powers are in [0, 1]; a power of 1.2 on a non-zero gradient is refused,
    on a zero gradient it is not evaluated and passes."""
    from cgfd3d_gb300 import _lib
    L = _lib.lib()
    z, m = _fixture()
    r = np.ascontiguousarray(m["rec"], np.float32)
    assert L.cgfd_media_layer_pow_ok(10, r.ctypes.data, r.size // 10) == 1
    r2 = r.copy()
    r2[1, 2, 3, 6] = 1.2                       # vp power, gradient 0.3-0.4 there
    assert L.cgfd_media_layer_pow_ok(10, r2.ctypes.data, r2.size // 10) == 0
    r3 = r.copy()
    r3[1, 2, 3, 9] = 1.2                       # vs power with its gradient zeroed
    r3[1, 2, 3, 8] = 0.0
    assert L.cgfd_media_layer_pow_ok(10, r3.ctypes.data, r3.size // 10) == 1


FIX_GRID = os.path.join(REPO, "tests", "golden", "media", "grid_el_iso.npz")


def _grid():
    from cgfd3d_gb300 import media
    z = np.load(FIX_GRID)
    g = np.load(FIX)
    return z, g, media.read_md3grd(bytes(z["md3grd"]).decode(), z["ext"])


@pytest.mark.parametrize("method", ["loc", "har", "ari"])
def test_oracle_grid_matches_reference_bitwise(method):
    """3-D grid models (media_grid2model_el_iso): three layers of three
    levels, coincident levels at a layer boundary, a boundary on a flat grid
    level, points below the last level; the reader's crop restated."""
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle
    z, g, m = _grid()
    assert (m["NI"], m["NL"], m["rec"].shape[-1]) == (9, 3, 4)
    got = oracle.grid_el_iso(m, g["x3d"], g["y3d"], g["z3d"], method)
    for a, k in zip(got, ("rho", "lam", "mu")):
        np.testing.assert_array_equal(a.view(np.int32), z[k + "_" + method].view(np.int32))


FIX_GRID_VTI = os.path.join(REPO, "tests", "golden", "media", "grid_el_vti.npz")
GRID_VTI_TYPES = ["elastic_vti_prem", "elastic_vti_thomsen", "elastic_vti_cij"]


def _grid_vti(kind):
    from cgfd3d_gb300 import media
    z = np.load(FIX_GRID_VTI)
    g = np.load(FIX)
    return z, g, media.read_md3grd(bytes(z[kind + "_md3grd"]).decode(), z["ext"])


@pytest.mark.parametrize("kind", GRID_VTI_TYPES)
def test_oracle_grid_vti_matches_reference_bitwise(kind):
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle
    z, g, m = _grid_vti(kind)
    assert m["media_type"] == kind and m["rec"].shape[-1] == 7
    got = oracle.grid_el_vti_loc(m, g["x3d"], g["y3d"], g["z3d"])
    for a, k in zip(got, VTI_OUT):
        np.testing.assert_array_equal(a.view(np.int32), z[kind + "_" + k].view(np.int32))


def test_har_and_ari_differ():
    z, _ = _fixture()
    d = z["lam_har"] != z["lam_ari"]
    assert d.sum() > 500


def test_oracle_refuses_points_outside_the_mesh():
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle
    z, m = _fixture()
    x = z["x3d"].copy()
    x[0, 0, 0] = m["MINX"] - 10.0
    assert oracle.layer_el_iso_loc(m, x, z["y3d"], z["z3d"]) is None


@pytest.mark.gpu
@pytest.mark.parametrize("method,sfx", METHODS)
def test_device_matches_reference(method, sfx):
    """Within 2e-6 relative: the device's double pow may differ from the
    host libm's in its last bit, which can move a float rounding."""
    from cgfd3d_gb300 import _lib, media
    z, m = _fixture()
    got = media.layer_el_iso(m, z["x3d"], z["y3d"], z["z3d"], method)
    for g, n in zip(got, ("lam", "mu", "rho")):
        np.testing.assert_allclose(g, z[n + sfx], rtol=2e-6, atol=0)
    x = z["x3d"].copy()
    x[0, 0, 0] = m["MINX"] - 10.0
    with pytest.raises(_lib.CgfdError):
        media.layer_el_iso(m, x, z["y3d"], z["z3d"], method)


REF = ref_tree() or ""


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "media")),
                    reason="reference tree not present")
@pytest.mark.parametrize("method,sfx", METHODS)
def test_dropin_adapter_inside_reference(method, sfx, tmp_path):
    """The media drop-in adapter runs inside the reference's process: the
    reference's media_layer2model_el_iso call is wrapped, the adapter reads
    the .md3lay with the reference's reader and hands its arrays to
    cgfd_media_layer_el_iso, answered here by the oracle (oracle/media_stub.c).
    The result must equal the reference's own bit for bit."""
    import struct
    import subprocess
    subprocess.run(["make", "-C", os.path.join(REPO, "oracle"), "-j8", "REF=" + REF,
                    "_ref/ref_probe_media"], check=True, capture_output=True)
    z, _ = _fixture()
    lay = tmp_path / "model.md3lay"
    lay.write_bytes(bytes(z["md3lay"]))
    nz, ny, nx = z["x3d"].shape
    grid = tmp_path / "grid.bin"
    with open(grid, "wb") as f:
        f.write(struct.pack("<3i", nx, ny, nz))
        for a in (z["x3d"], z["y3d"], z["z3d"]):
            f.write(np.ascontiguousarray(a, "<f4").tobytes())
    out = tmp_path / "out.bin"
    exe = os.path.join(REPO, "oracle", "_ref", "ref_probe_media")
    r = subprocess.run([exe, "layer", str(lay), str(grid), method, str(out)],
                       capture_output=True, text=True, check=True)
    assert "discretising the layered model on the GPU (method %s)" % method in r.stdout
    got = np.fromfile(out, "<f4").reshape(3, nz, ny, nx)
    for g, n in zip(got, ("lam", "mu", "rho")):
        np.testing.assert_array_equal(g.view(np.int32), z[n + sfx].view(np.int32))
    # another method goes to the reference's routine, which rejects it
    r = subprocess.run([exe, "layer", str(lay), str(grid), "tti", str(out)],
                       capture_output=True, text=True)
    assert r.returncode == 1 and "Wrong parametrization method" in r.stderr


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "media")),
                    reason="reference tree not present")
@pytest.mark.parametrize("kind,method", VTI_CASES)
def test_dropin_adapter_vti_inside_reference(kind, method, tmp_path):
    """As test_dropin_adapter_inside_reference, for media_layer2model_el_vti."""
    import struct
    import subprocess
    subprocess.run(["make", "-C", os.path.join(REPO, "oracle"), "-j8", "REF=" + REF,
                    "_ref/ref_probe_media"], check=True, capture_output=True)
    z, _ = _vti(kind)
    lay = tmp_path / "model.md3lay"
    lay.write_bytes(bytes(z[kind + "_md3lay"]))
    nz, ny, nx = z["x3d"].shape
    grid = tmp_path / "grid.bin"
    with open(grid, "wb") as f:
        f.write(struct.pack("<3i", nx, ny, nz))
        for a in (z["x3d"], z["y3d"], z["z3d"]):
            f.write(np.ascontiguousarray(a, "<f4").tobytes())
    out = tmp_path / "out.bin"
    exe = os.path.join(REPO, "oracle", "_ref", "ref_probe_media")
    r = subprocess.run([exe, "layer_vti", str(lay), str(grid), method, str(out)],
                       capture_output=True, text=True, check=True)
    assert "discretising the layered model on the GPU (method %s)" % method in r.stdout
    got = np.fromfile(out, "<f4").reshape(6, nz, ny, nx)
    for g, n in zip(got, VTI_OUT):
        np.testing.assert_array_equal(g.view(np.int32), z["%s_%s_%s" % (kind, method, n)]
                                      .view(np.int32))


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "media")),
                    reason="reference tree not present")
@pytest.mark.parametrize("vis", [False, True])
def test_dropin_adapter_bin_inside_reference(vis, tmp_path):
    """The adapter takes the reference's media_bin2model_el_iso / _vis_iso
    calls: whole-file reads, library call (answered by the oracle here),
    the reference's values bit for bit."""
    import subprocess
    subprocess.run(["make", "-C", os.path.join(REPO, "oracle"), "-j8", "REF=" + REF,
                    "_ref/ref_probe_media"], check=True, capture_output=True)
    z = np.load(FIX_BIN)
    g = np.load(FIX)
    nz, ny, nx = g["x3d"].shape
    grid = tmp_path / "grid.bin"
    with open(grid, "wb") as f:
        f.write(np.array([nx, ny, nz], "<i4").tobytes())
        for a in (g["x3d"], g["y3d"], g["z3d"]):
            f.write(np.ascontiguousarray(a, "<f4").tobytes())
    params = tmp_path / "params.bin"
    with open(params, "wb") as f:
        for k, t in (("order", "<i4"), ("size", "<i4"), ("spacing", "<f4"), ("origin", "<f4"),
                     ("ext", "<f4")):
            f.write(np.ascontiguousarray(z[k], t).tobytes())
    keys = ("qp_vol", "qs_vol") if vis else ("rho_vol", "vp_vol", "vs_vol")
    files = []
    for k in keys:
        files.append(str(tmp_path / (k + ".bin")))
        np.ascontiguousarray(z[k], "<f4").tofile(files[-1])
    out = tmp_path / "out.bin"
    exe = os.path.join(REPO, "oracle", "_ref", "ref_probe_media")
    r = subprocess.run([exe, "bin_vis" if vis else "bin", str(grid), str(params)] + files +
                       [str(out)], capture_output=True, text=True, check=True)
    assert "discretising the binary model on the GPU" in r.stdout
    got = np.fromfile(out, "<f4").reshape(len(keys), nz, ny, nx)
    for a, k in zip(got, ("Qp", "Qs") if vis else ("rho", "lam", "mu")):
        np.testing.assert_array_equal(a.view(np.int32), z[k].view(np.int32))


@pytest.mark.gpu
@pytest.mark.parametrize("vis", [False, True])
def test_device_bin_matches_reference(vis):
    """Trilinear interpolation in the reference's float order (--fmad=false):
    bit for bit; lambda within a float rounding of the double form."""
    from cgfd3d_gb300 import media
    z = np.load(FIX_BIN)
    g = np.load(FIX)
    lay = media.BinModel.of(z["order"], z["size"], z["spacing"], z["origin"])
    keys = ("qp_vol", "qs_vol") if vis else ("rho_vol", "vp_vol", "vs_vol")
    got = media.bin_model(lay, z["ext"], [z[k] for k in keys], g["x3d"], g["y3d"], g["z3d"],
                          vis)
    for a, k in zip(got, ("Qp", "Qs") if vis else ("rho", "lam", "mu")):
        np.testing.assert_array_equal(a.view(np.int32), z[k].view(np.int32))
    bad = media.BinModel.of(z["order"], z["size"], z["spacing"], z["origin"])
    bad.origin[1] = float(g["x3d"].max()) + 10.0          # model east of the grid
    with pytest.raises(Exception):
        media.bin_model(bad, z["ext"], [z[k] for k in keys], g["x3d"], g["y3d"], g["z3d"], vis)


@pytest.mark.gpu
@pytest.mark.parametrize("vis", [False, True])
def test_device_bin_box_equals_whole_files(vis):
    """Volumes holding only the crop's box of the files (what a caller that
    reads just the box passes) give the whole-file results bit for bit; a
    box that misses part of the crop is refused."""
    from cgfd3d_gb300 import media
    z = np.load(FIX_BIN)
    g = np.load(FIX)
    lay = media.BinModel.of(z["order"], z["size"], z["spacing"], z["origin"])
    keys = ("qp_vol", "qs_vol") if vis else ("rho_vol", "vp_vol", "vs_vol")
    first, count = media.bin_crop(lay, z["ext"], g["z3d"])
    size = [int(v) for v in z["size"]]
    assert any(c < s for c, s in zip(count, size))        # a real crop
    cut = tuple(slice(f, f + c) for f, c in zip(first[::-1], count[::-1]))
    boxes = [np.asarray(z[k], np.float32).reshape(size[::-1])[cut] for k in keys]
    whole = media.bin_model(lay, z["ext"], [z[k] for k in keys], g["x3d"], g["y3d"], g["z3d"],
                            vis)
    got = media.bin_model_box(lay, z["ext"], (first, count), boxes, g["x3d"], g["y3d"],
                              g["z3d"], vis)
    for a, b in zip(got, whole):
        np.testing.assert_array_equal(a.view(np.int32), b.view(np.int32))
    short = (first, tuple(c - 1 if d == 0 else c for d, c in enumerate(count)))
    cut2 = tuple(slice(f, f + c) for f, c in zip(short[0][::-1], short[1][::-1]))
    small = [np.asarray(z[k], np.float32).reshape(size[::-1])[cut2] for k in keys]
    with pytest.raises(Exception):
        media.bin_model_box(lay, z["ext"], short, small, g["x3d"], g["y3d"], g["z3d"], vis)


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "media")),
                    reason="reference tree not present")
@pytest.mark.parametrize("method", ["loc", "har", "ari"])
def test_dropin_adapter_grid_inside_reference(method, tmp_path):
    """The adapter takes media_grid2model_el_iso: the reference's reader and
    crop, then the library call (answered by the oracle here)."""
    import subprocess
    subprocess.run(["make", "-C", os.path.join(REPO, "oracle"), "-j8", "REF=" + REF,
                    "_ref/ref_probe_media"], check=True, capture_output=True)
    z, g, _ = _grid()
    grd = tmp_path / "model.md3grd"
    grd.write_bytes(bytes(z["md3grd"]))
    nz, ny, nx = g["x3d"].shape
    grid = tmp_path / "grid.bin"
    with open(grid, "wb") as f:
        f.write(np.array([nx, ny, nz], "<i4").tobytes())
        for a in (g["x3d"], g["y3d"], g["z3d"]):
            f.write(np.ascontiguousarray(a, "<f4").tobytes())
    ext = tmp_path / "ext.bin"
    np.ascontiguousarray(z["ext"], "<f4").tofile(ext)
    out = tmp_path / "out.bin"
    exe = os.path.join(REPO, "oracle", "_ref", "ref_probe_media")
    r = subprocess.run([exe, "grid", str(grd), str(grid), method, str(ext), str(out)],
                       capture_output=True, text=True, check=True)
    # loc goes to the library; har and ari stay with the reference's routine
    on_gpu = "discretising the grid model on the GPU (method %s)" % method in r.stdout
    assert on_gpu == (method == "loc")
    got = np.fromfile(out, "<f4").reshape(3, nz, ny, nx)
    for a, k in zip(got, ("rho", "lam", "mu")):
        np.testing.assert_array_equal(a.view(np.int32), z[k + "_" + method].view(np.int32))


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "media")),
                    reason="reference tree not present")
@pytest.mark.parametrize("kind", GRID_VTI_TYPES)
def test_dropin_adapter_grid_vti_inside_reference(kind, tmp_path):
    import subprocess
    subprocess.run(["make", "-C", os.path.join(REPO, "oracle"), "-j8", "REF=" + REF,
                    "_ref/ref_probe_media"], check=True, capture_output=True)
    z, g, _ = _grid_vti(kind)
    grd = tmp_path / "model.md3grd"
    grd.write_bytes(bytes(z[kind + "_md3grd"]))
    nz, ny, nx = g["x3d"].shape
    grid = tmp_path / "grid.bin"
    with open(grid, "wb") as f:
        f.write(np.array([nx, ny, nz], "<i4").tobytes())
        for a in (g["x3d"], g["y3d"], g["z3d"]):
            f.write(np.ascontiguousarray(a, "<f4").tobytes())
    ext = tmp_path / "ext.bin"
    np.ascontiguousarray(z["ext"], "<f4").tofile(ext)
    out = tmp_path / "out.bin"
    exe = os.path.join(REPO, "oracle", "_ref", "ref_probe_media")
    r = subprocess.run([exe, "grid_vti", str(grd), str(grid), "loc", str(ext), str(out)],
                       capture_output=True, text=True, check=True)
    assert "discretising the grid model on the GPU (method loc)" in r.stdout
    got = np.fromfile(out, "<f4").reshape(6, nz, ny, nx)
    for a, k in zip(got, VTI_OUT):
        np.testing.assert_array_equal(a.view(np.int32), z[kind + "_" + k].view(np.int32))


@pytest.mark.gpu
@pytest.mark.parametrize("kind", GRID_VTI_TYPES)
def test_device_grid_vti_matches_reference(kind):
    """VTI grid models with loc on the device: bit for bit (no pow here; the
    double arithmetic of para2vti is kept)."""
    from cgfd3d_gb300 import media
    z, g, m = _grid_vti(kind)
    got = media.grid_el_vti(m, g["x3d"], g["y3d"], g["z3d"])
    for a, k in zip(got, VTI_OUT):
        np.testing.assert_array_equal(a.view(np.int32), z[kind + "_" + k].view(np.int32))


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "media")),
                    reason="reference tree not present")
@pytest.mark.parametrize("case", [("iso", "har"), ("iso", "loc"), ("elastic_vti_thomsen", "ari"),
                                  ("elastic_vti_cij", "loc")])
def test_dropin_adapter_aniso_inside_reference(case, tmp_path):
    """media_layer2model_el_aniso for isotropic and VTI layered models: the
    adapter's build (library call answered by the oracle, then the spreading
    into the 21 constants) against the unmodified reference, all 22 volumes
    bit for bit."""
    import subprocess
    subprocess.run(["make", "-C", os.path.join(REPO, "oracle"), "-j8", "REF=" + REF,
                    "_ref/ref_probe", "_ref/ref_probe_media"], check=True, capture_output=True)
    kind, method = case
    if kind == "iso":
        z, _ = _fixture()
        text, grid_src = bytes(z["md3lay"]), z
    else:
        z, _ = _vti(kind)
        text, grid_src = bytes(z[kind + "_md3lay"]), z
    lay = tmp_path / "model.md3lay"
    lay.write_bytes(text)
    nz, ny, nx = grid_src["x3d"].shape
    grid = tmp_path / "grid.bin"
    with open(grid, "wb") as f:
        f.write(np.array([nx, ny, nz], "<i4").tobytes())
        for a in (grid_src["x3d"], grid_src["y3d"], grid_src["z3d"]):
            f.write(np.ascontiguousarray(a, "<f4").tobytes())
    outs = []
    for exe in ("ref_probe", "ref_probe_media"):
        out = tmp_path / (exe + ".bin")
        r = subprocess.run([os.path.join(REPO, "oracle", "_ref", exe), "layer_aniso", str(lay),
                            str(grid), method, str(out)], capture_output=True, text=True,
                           check=True)
        outs.append(np.fromfile(out, "<f4").reshape(22, nz, ny, nx))
    assert "discretising the layered model on the GPU (method %s)" % method in r.stdout
    np.testing.assert_array_equal(outs[1].view(np.int32), outs[0].view(np.int32))


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "media")),
                    reason="reference tree not present")
@pytest.mark.parametrize("kind", ["elastic_isotropic", "elastic_vti_prem"])
def test_dropin_adapter_grid_aniso_inside_reference(kind, tmp_path):
    """media_grid2model_el_aniso for isotropic and VTI grid models with loc:
    the adapter's build against the unmodified reference, 22 volumes bit for
    bit."""
    import subprocess
    subprocess.run(["make", "-C", os.path.join(REPO, "oracle"), "-j8", "REF=" + REF,
                    "_ref/ref_probe", "_ref/ref_probe_media"], check=True, capture_output=True)
    if kind == "elastic_isotropic":
        z, g, _ = _grid()
        text = bytes(z["md3grd"])
    else:
        z, g, _ = _grid_vti(kind)
        text = bytes(z[kind + "_md3grd"])
    grd = tmp_path / "model.md3grd"
    grd.write_bytes(text)
    nz, ny, nx = g["x3d"].shape
    grid = tmp_path / "grid.bin"
    with open(grid, "wb") as f:
        f.write(np.array([nx, ny, nz], "<i4").tobytes())
        for a in (g["x3d"], g["y3d"], g["z3d"]):
            f.write(np.ascontiguousarray(a, "<f4").tobytes())
    ext = tmp_path / "ext.bin"
    np.ascontiguousarray(z["ext"], "<f4").tofile(ext)
    outs = []
    for exe in ("ref_probe", "ref_probe_media"):
        out = tmp_path / (exe + ".bin")
        r = subprocess.run([os.path.join(REPO, "oracle", "_ref", exe), "grid_aniso", str(grd),
                            str(grid), "loc", str(ext), str(out)], capture_output=True,
                           text=True, check=True)
        outs.append(np.fromfile(out, "<f4").reshape(22, nz, ny, nx))
    assert "discretising the grid model on the GPU (method loc)" in r.stdout
    np.testing.assert_array_equal(outs[1].view(np.int32), outs[0].view(np.int32))


@pytest.mark.gpu
def test_device_grid_matches_reference():
    """loc on the device in the reference's float order (--fmad=false, no
    pow on this path): bit for bit.  har and ari are refused."""
    from cgfd3d_gb300 import _lib, media
    z, g, m = _grid()
    got = media.grid_el_iso(m, g["x3d"], g["y3d"], g["z3d"], "loc")
    for a, k in zip(got, ("rho", "lam", "mu")):
        np.testing.assert_array_equal(a.view(np.int32), z[k + "_loc"].view(np.int32))
    for method in ("har", "ari"):
        with pytest.raises(_lib.CgfdError):
            media.grid_el_iso(m, g["x3d"], g["y3d"], g["z3d"], method)


@pytest.mark.gpu
@pytest.mark.parametrize("kind,method", VTI_CASES)
def test_device_vti_matches_reference(kind, method):
    """Within 2e-6 relative (the device's double pow and the reference's)."""
    from cgfd3d_gb300 import media
    z, m = _vti(kind)
    got = media.layer_el_vti(m, z["x3d"], z["y3d"], z["z3d"], method)
    for g, n in zip(got, VTI_OUT):
        np.testing.assert_allclose(g, z["%s_%s_%s" % (kind, method, n)], rtol=2e-6, atol=0)


@pytest.mark.gpu
def test_device_refuses_unknown_method():
    from cgfd3d_gb300 import _lib, media
    z, m = _fixture()
    with pytest.raises(_lib.CgfdError):
        media.layer_el_iso(m, z["x3d"], z["y3d"], z["z3d"], "vol")


@pytest.mark.gpu
@pytest.mark.parametrize("method", ["har", "ari"])
def test_device_matches_oracle_larger(method):
    """A larger grid (bench model generator, 64 x 56 x 40 cells) against the
    oracle: the same points averaged, values within float rounding."""
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle
    from types import SimpleNamespace
    from cgfd3d_gb300 import media, models
    ni, nj, nk = 64, 56, 40
    shp = (nk + 6, nj + 6, ni + 6)
    X, Y, Z = [a.reshape(shp) for a in
               models._coords_of(SimpleNamespace(ni=ni, nj=nj, nk=nk), 2024)]
    m = _bench_model(X, Y, Z)
    want = oracle.layer_el_iso(m, X, Y, Z, method)
    loc = oracle.layer_el_iso(m, X, Y, Z, "loc")
    got = media.layer_el_iso(m, X, Y, Z, method)
    assert (want[0] != loc[0]).sum() > 1000
    for g, w in zip(got, want):
        np.testing.assert_allclose(g, w, rtol=2e-6, atol=0)


def _bench_model(X, Y, Z):
    """Four interfaces spread over the grid's depth, gradients with powers."""
    rng = np.random.default_rng(3)
    NX, NY = 30, 24
    minx, miny = float(X.min()) - 10.0, float(Y.min()) - 10.0
    dx = (float(X.max()) + 10.0 - minx) / (NX - 1)
    dy = (float(Y.max()) + 10.0 - miny) / (NY - 1)
    XX, YY = np.meshgrid(minx + dx * np.arange(NX), miny + dy * np.arange(NY))
    zmin, zmax = float(Z.min()), float(Z.max())
    recs = []
    for n in range(4):
        t = zmax - (0.1 + 0.25 * n) * (zmax - zmin)
        e = t + 0.03 * (zmax - zmin) * np.sin(XX / (0.3 * (dx * NX)) + n)
        r = lambda a: a * (1 + 0.02 * rng.uniform(-1, 1, XX.shape))
        recs.append(np.stack([e, r(2300 + 150 * n), np.full_like(XX, 0.01), np.full_like(XX, 1.0),
                              r(4000 + 700 * n), np.full_like(XX, 0.04), np.full_like(XX, 0.9),
                              r(2300 + 400 * n), np.full_like(XX, 0.0), np.full_like(XX, 1.0)],
                             -1))
    return dict(NI=4, NX=NX, NY=NY, MINX=minx, MINY=miny, DX=dx, DY=dy,
                rec=np.stack(recs).astype(np.float32))
