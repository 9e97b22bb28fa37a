"""The C ABI library loads, exports every entry point include/plenoxels_gb300.h declares,
has the struct layout the header defines, and rejects bad arguments before touching a
GPU. CPU only (no kernel is launched)."""
import ctypes
import os
import re
import subprocess
import tempfile

import numpy as np
import pytest

from plenoxels_gb300 import _lib
from oracle import hash as ohash

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "plenoxels_gb300.h")


def _declared():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(pgb_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol(lib):
    names = _declared()
    assert len(names) >= 20
    for n in names:
        assert hasattr(lib, n), f"{n} declared in the header but not exported"
    assert set(names) == set(_lib.symbols()), "ctypes binding and header disagree"


def test_struct_layout_matches_header(tmp_path):
    src = tmp_path / "layout.c"
    src.write_text(
        '#include <stddef.h>\n#include <stdio.h>\n#include "plenoxels_gb300.h"\n'
        "int main(void){\n"
        'printf("%zu %zu %zu %zu %zu\\n", sizeof(pgb_grid), offsetof(pgb_grid, origin),'
        " offsetof(pgb_grid, points_distance), offsetof(pgb_grid, clip), offsetof(pgb_grid, mode));\n"
        'printf("%zu %zu %zu %zu\\n", sizeof(pgb_cameras), offsetof(pgb_cameras, camera_angle_x),'
        " offsetof(pgb_cameras, near), offsetof(pgb_cameras, seed));\n"
        'printf("%zu %zu %zu %zu %zu %zu %zu %zu %zu %zu\\n", sizeof(pgb_rays), offsetof(pgb_rays, num_rays),'
        " offsetof(pgb_rays, delta_step), offsetof(pgb_rays, seed), offsetof(pgb_rays, term_threshold),"
        " offsetof(pgb_rays, background), offsetof(pgb_rays, log_transmittance),"
        " offsetof(pgb_rays, chunk_samples), offsetof(pgb_rays, first_ray),"
        " offsetof(pgb_rays, grad_marks));\n"
        'printf("%zu %zu %zu %zu %zu\\n", sizeof(pgb_scene), offsetof(pgb_scene, dims),'
        " offsetof(pgb_scene, origin), offsetof(pgb_scene, num_samples), offsetof(pgb_scene, delta_step));\n"
        "return 0;}\n")
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-I", os.path.dirname(HEADER), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split("\n")
    g = list(map(int, out[0].split()))
    c = list(map(int, out[1].split()))
    r = list(map(int, out[2].split()))
    G, C, R = _lib.PgbGrid, _lib.PgbCameras, _lib.PgbRays
    assert g == [ctypes.sizeof(G), G.origin.offset, G.points_distance.offset, G.clip.offset, G.mode.offset]
    assert c == [ctypes.sizeof(C), C.camera_angle_x.offset, C.near.offset, C.seed.offset]
    assert r == [ctypes.sizeof(R), R.num_rays.offset, R.delta_step.offset, R.seed.offset,
                 R.term_threshold.offset, R.background.offset, R.log_transmittance.offset,
                 R.chunk_samples.offset, R.first_ray.offset, R.grad_marks.offset]
    sc = list(map(int, out[3].split()))
    P = _lib.PgbScene
    assert sc == [ctypes.sizeof(P), P.dims.offset, P.origin.offset, P.num_samples.offset,
                  P.delta_step.offset]


def test_host_hash_matches_oracle(lib):
    rng = np.random.default_rng(0)
    for _ in range(200):
        seed = int(rng.integers(0, 2 ** 63))
        a = int(rng.integers(0, 2 ** 40))
        b = int(rng.integers(0, 2 ** 20))
        assert lib.pgb_hash_uniform(seed, a, b) == float(ohash.uniform(seed, a, b))
    j = ohash.stratified_jitter(5, 3, 7)
    for r in range(3):
        for s in range(7):
            assert lib.pgb_hash_uniform(5, r, s) == float(j[r, s])
    assert j.min() >= 0 and j.max() < 1


def test_status_strings_and_version(lib):
    assert b"sm_103a" in lib.pgb_version()
    assert lib.pgb_status_string(0) == b"ok"
    assert lib.pgb_status_string(-1) == b"invalid argument"
    assert lib.pgb_train_workspace_bytes() >= 8 * 8192
    # one mark bit per 4-cell unit of the gradient
    assert [lib.pgb_mark_words(n) for n in (0, 1, 128, 129, 256 ** 3)] == [0, 1, 1, 2, 256 ** 3 // 128]


def test_argument_validation_without_launch(lib):
    before = lib.pgb_launch_count()
    g = _lib.PgbGrid()
    r = _lib.PgbRays()
    # null grid
    assert lib.pgb_render_fwd(None, ctypes.byref(r), 16, None) == _lib.PGB_ERR_ARG
    # bad dtype / dims / alignment
    g.cells = 256
    g.dtype = 7
    g.dims[0] = g.dims[1] = g.dims[2] = 4
    assert lib.pgb_render_fwd(ctypes.byref(g), ctypes.byref(r), 16, None) == _lib.PGB_ERR_ARG
    g.dtype = _lib.PGB_F32
    g.mode = 5
    assert lib.pgb_render_fwd(ctypes.byref(g), ctypes.byref(r), 16, None) == _lib.PGB_ERR_ARG
    g.mode = _lib.PGB_TRILINEAR
    g.cells = 260  # not 16-byte aligned
    assert lib.pgb_render_fwd(ctypes.byref(g), ctypes.byref(r), 16, None) == _lib.PGB_ERR_ALIGN
    g.cells = 256
    r.num_rays = 4
    r.num_samples = 10 ** 6
    assert lib.pgb_render_fwd(ctypes.byref(g), ctypes.byref(r), 16, None) == _lib.PGB_ERR_UNSUPPORTED
    r.num_samples = 8
    # the log-sum transmittance needs clipped fp32/BF16 cells
    r.log_transmittance = 1
    g.clip = 0
    assert lib.pgb_render_fwd(ctypes.byref(g), ctypes.byref(r), 16, None) == _lib.PGB_ERR_ARG
    g.clip = 1
    g.dtype = _lib.PGB_F64
    g.cells = 512
    assert lib.pgb_render_fwd(ctypes.byref(g), ctypes.byref(r), 16, None) == _lib.PGB_ERR_UNSUPPORTED
    g.dtype = _lib.PGB_F32
    g.cells = 256
    r.log_transmittance = 0
    assert lib.pgb_render_fwd(ctypes.byref(g), ctypes.byref(r), 16, None) == _lib.PGB_ERR_ARG  # no rays
    assert lib.pgb_render_train(ctypes.byref(g), ctypes.byref(r), None, 1.0, None, None, None, None,
                                None) == _lib.PGB_ERR_ARG
    assert lib.pgb_wrap_indices(None, 3, None, None) == _lib.PGB_ERR_ARG
    assert lib.pgb_fill_zero(24, 16, None) == _lib.PGB_ERR_ALIGN
    assert lib.pgb_clear_marked(16, 8, 64, 16, None) == _lib.PGB_ERR_ARG  # cell bytes
    assert lib.pgb_clear_marked(None, 16, 64, 16, None) == _lib.PGB_ERR_ARG
    assert lib.pgb_clear_marked(24, 16, 64, 16, None) == _lib.PGB_ERR_ALIGN
    # even_spread with a non-square ray count
    assert lib.pgb_generate_rays(16, 1, 10, ctypes.c_float(0.5), 16, 4, 4, None, 1, 16, 16, None,
                                 None) == _lib.PGB_ERR_ARG
    assert lib.pgb_launch_count() == before, "validation failures must not launch kernels"


def test_operators_reject_cpu_tensors():
    import torch
    import plenoxels_gb300 as pg
    grid = torch.zeros(4, 4, 4, 4)
    with pytest.raises(ValueError):
        pg.get_nearest_voxels(torch.zeros(3, 3), grid)
    with pytest.raises(ValueError):
        pg.render_rays(grid, torch.zeros(2, 3), torch.zeros(2, 3), 0.1, 8, 0.25)
    with pytest.raises(ValueError):
        pg.generate_grid(4, 4, 4, device="cpu")
    with pytest.raises(ValueError):
        pg.compute_alpha_weighted_pixels(torch.zeros(1, 2, 3, 4))


def test_probe_helper_loads_and_validates_arguments():
    """The device-memory probes live in their own helper library (not the renderer's ABI):
    it loads and rejects bad arguments without launching anything."""
    from plenoxels_gb300 import probes
    p = probes.load()
    assert p.pgb_probe_random_reads(None, 256, 8, 1, 16, None) == _lib.PGB_ERR_ARG
    assert p.pgb_probe_random_reads(24, 256, 8, 1, 16, None) == _lib.PGB_ERR_ALIGN
    assert p.pgb_probe_random_atomics(16, 8, 8, 1, None) == _lib.PGB_ERR_ARG  # < one slot
    assert p.pgb_probe_random_atomics(16, 256, 0, 1, None) == _lib.PGB_OK  # nothing to do
    assert not any(n.startswith("pgb_probe") for n in _declared())
