"""Image to density (image_to_pl_function, include/MA/functions.hpp:82-120): the PGM
reader, the vertex grid and values, and the C ABI's ma_mesh_create_image."""
import numpy as np
import pytest

from mongeampere_gb300.mesh import image_grid, read_pgm


def _image(seed=0, w=7, h=5):
    return np.random.default_rng(seed).integers(0, 256, size=(h, w)).astype(np.float64)


def test_pgm_reader_binary_and_text(tmp_path):
    img = _image()
    h, w = img.shape
    p5 = tmp_path / "a.pgm"
    p5.write_bytes(b"P5\n# a comment\n%d %d\n255\n" % (w, h) + img.astype(np.uint8).tobytes())
    p2 = tmp_path / "b.pgm"
    p2.write_text("P2\n%d %d\n255\n" % (w, h) + " ".join(str(int(v)) for v in img.ravel()) + "\n")
    np.testing.assert_array_equal(read_pgm(p5), img)
    np.testing.assert_array_equal(read_pgm(p2), img)


def test_image_grid_matches_the_reference_formula():
    img = _image(1)
    h, w = img.shape
    m = image_grid(img)
    # vertex (i, j) at (-1 + 2 i / (w - 1), -1 + 2 j / (h - 1)) with image(i, h - j - 1) / 255 + 1e-3
    for i in range(w):
        for j in range(h):
            assert m.gx[i] == pytest.approx(-1 + 2 * i / (w - 1), abs=1e-15)
            assert m.gy[j] == pytest.approx(-1 + 2 * j / (h - 1), abs=1e-15)
            assert m.values[j, i] == img[h - j - 1, i] / 255.0 + 1e-3


@pytest.mark.gpu
def test_create_image_mesh_through_the_abi():
    import ctypes
    from mongeampere_gb300 import api
    from mongeampere_gb300 import _lib as L
    img = _image(2, 33, 17)
    ctx = api.Context(0)
    h = ctypes.c_void_p()
    px = np.ascontiguousarray(img)
    st = ctx.lib.ma_mesh_create_image(ctx.h, 33, 17, px.ctypes.data_as(L._dp), ctypes.byref(h))
    assert st == 0
    tot = ctypes.c_double()
    assert ctx.lib.ma_mesh_total_mass(h, ctypes.byref(tot)) == 0
    assert tot.value == pytest.approx(image_grid(img).total_mass(), rel=1e-13)
    ctx.lib.ma_mesh_destroy(h)
