"""The C ABI without a GPU: the library loads, exports every symbol include/sdfb.h declares, its
structs have the header's layout, and its host-only entry points match the reference."""
from __future__ import annotations

import ctypes as C
import os
import re
import subprocess

import numpy as np
import pytest

from conftest import ROOT

HEADER = os.path.join(ROOT, "include", "sdfb.h")


def declared_functions() -> list[str]:
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(sdfb_\w+)\s*\(", text)))


def test_exports_every_declared_symbol(lib):
    names = declared_functions()
    assert len(names) >= 10
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, f"declared in include/sdfb.h but not exported: {missing}"


def test_bindings_cover_the_header(lib):
    import sdfb
    assert set(declared_functions()) <= set(sdfb.SIGNATURES)


def test_struct_layout_matches_header(tmp_path):
    import sdfb
    src = tmp_path / "sizes.c"
    src.write_text('#include <stdio.h>\n#include <stddef.h>\n#include "sdfb.h"\n'
                   'int main(void){printf("%zu %zu %zu %zu %zu\\n", sizeof(sdfb_grid_desc), sizeof(sdfb_opts),'
                   ' sizeof(sdfb_stats), offsetof(sdfb_stats, voxels), offsetof(sdfb_opts, count_work));return 0;}\n')
    exe = tmp_path / "sizes"
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()
    assert int(out[0]) == C.sizeof(sdfb.GridDesc)
    assert int(out[1]) == C.sizeof(sdfb.Opts)
    assert int(out[2]) == C.sizeof(sdfb.Stats)
    assert int(out[3]) == sdfb.Stats.voxels.offset
    assert int(out[4]) == sdfb.Opts.count_work.offset


def test_material_struct_layout_matches_header(tmp_path):
    import sdfb
    src = tmp_path / "msizes.c"
    src.write_text('#include <stdio.h>\n#include <stddef.h>\n#include "sdfb.h"\n'
                   'int main(void){printf("%zu %zu %zu %zu %zu %zu\\n", sizeof(sdfb_texture), sizeof(sdfb_material),'
                   ' sizeof(sdfb_materials), offsetof(sdfb_materials, uvs), offsetof(sdfb_materials, num_textures),'
                   ' offsetof(sdfb_material, base_color_texture));return 0;}\n')
    exe = tmp_path / "msizes"
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    out = [int(x) for x in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()]
    assert out == [C.sizeof(sdfb.Texture), C.sizeof(sdfb.Material), C.sizeof(sdfb.Materials),
                   sdfb.Materials.uvs.offset, sdfb.Materials.num_textures.offset,
                   sdfb.Material.base_color_texture.offset]


def test_abi_version(lib):
    assert lib.sdfb_abi_version() == 1


def test_grid_sizing_host(golden, lib):
    import sdfb
    for row in golden["grid_sizing_cases"]:
        g = sdfb.grid_from_bounds_res(row[0:3], row[3:6], int(row[6]))
        assert [np.float32(x) for x in g.origin] == [np.float32(x) for x in row[7:10]]
        assert np.float32(g.voxel_size) == np.float32(row[10])
        assert (g.nx, g.ny, g.nz) == tuple(int(x) for x in row[11:14])


def test_weld_and_watertight_host(golden, lib):
    import sdfb
    w, n = sdfb.weld(golden["sphere1_soup"], (-1,) * 3, (1,) * 3)
    assert np.array_equal(w, golden["sphere1_weld"])
    assert sdfb.is_watertight(w)[0]
    cube = golden["cube_soup"]
    wh, _ = sdfb.weld(cube[:-6], (0, 0, 0), (1, 1, 1))
    ok, b, m = sdfb.is_watertight(wh)
    assert not ok and b == 4 and m == 0


def test_weld_matches_reference_on_generated_meshes(reference, lib):
    import sdfb
    from sdfb import meshgen as mg
    v, f = mg.displaced_icosphere(3, 0.35, 5)
    soup = v[f.reshape(-1)]
    lo, hi = soup.min(0), soup.max(0)
    w_ref, n_ref = reference.weld(soup, lo, hi)
    w, n = sdfb.weld(soup, lo, hi)
    assert n == n_ref and np.array_equal(w, w_ref)
    wm, nm = mg.weld(soup, lo, hi)
    assert np.array_equal(wm.shape[0], n_ref) and np.array_equal(nm.reshape(-1), w_ref)


def test_context_without_gpu_reports_no_device(lib):
    import sdfb
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    with pytest.raises(sdfb.SdfbError) as e:
        sdfb.Context(0)
    assert e.value.status == sdfb.ERR_NO_DEVICE
