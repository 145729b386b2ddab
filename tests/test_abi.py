"""CPU tests of the C ABI boundary: the library loads, exports every function
include/gg.h declares, validates options on the host and reports errors as
status codes (no GPU calls here beyond what fails cleanly without one)."""
import ctypes
import os
import re

import numpy as np
import pytest

import gpugrid as gg
import synth
from helpers import ROOT


def header_functions():
    src = open(os.path.join(ROOT, "include", "gg.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(?:int|const char \*)\s*\*?\s*(gg_\w+)\s*\(", src)))


def test_library_exports_every_declared_symbol():
    names = header_functions()
    assert len(names) >= 18, names
    lib = ctypes.CDLL(gg.LIB_PATH)
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_grid_gpu_header_compiles_as_drop_in(tmp_path):
    """A reference-style caller (grid.cu:481) builds unchanged against
    include/grid_gpu.cuh and links libgg.so, for all three instantiations."""
    import shutil
    import subprocess
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("no g++")
    src = tmp_path / "caller.cpp"
    src.write_text(r'''
#define __MOVING_WINDOW
#define POLARIZATIONS 1
#define GCF_GRID 8
#include "grid_gpu.cuh"
#include <vector>
int main() {
  std::vector<double2> o(100), i(4), v(4), g(64 * 16);
  std::vector<float2> fo(100), fi(4), fv(4), fg(64 * 16);
  gridGPU(o.data(), i.data(), v.data(), 4, 8, g.data(), 4);
  int a = gg_last_status();
  gridGPU(o.data(), fi.data(), fv.data(), 4, 8, fg.data(), 4);
  gridGPU(fo.data(), fi.data(), fv.data(), 4, 8, fg.data(), 4);
  return a == GG_OK ? 0 : 3;
}
''')
    exe = tmp_path / "caller"
    cuda_inc = "/usr/local/cuda/include"
    r = subprocess.run([gxx, "-std=c++14", str(src), "-o", str(exe),
                        "-I", os.path.join(ROOT, "include"), "-I", cuda_inc,
                        os.path.abspath(gg.LIB_PATH),
                        "-Wl,-rpath," + os.path.dirname(os.path.abspath(gg.LIB_PATH))],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    import torch
    if not torch.cuda.is_available():
        # without a GPU the call must fail with a status, not crash
        r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
        assert r.returncode == 3 and "gridGPU:" in r.stderr


def test_struct_layouts_match_header(tmp_path):
    """ctypes mirrors of the ABI structs have the C sizes and field offsets."""
    import shutil
    import subprocess
    cc = shutil.which("gcc")
    if not cc:
        pytest.skip("no gcc")
    structs = {"gg_options": gg.gg_options, "gg_job": gg.gg_job,
               "gg_request": gg.gg_request, "gg_result": gg.gg_result,
               "gg_server_config": gg.gg_server_config,
               "gg_server_stats": gg.gg_server_stats}
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "gg.h"', 'int main(void){']
    for name, cls in structs.items():
        lines.append(f'printf("{name} %zu\\n", sizeof({name}));')
        for fname, _ in cls._fields_:
            lines.append(f'printf("{name}.{fname} %zu\\n", offsetof({name}, {fname}));')
    lines.append("return 0;}")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    r = subprocess.run([cc, "-std=c99", str(src), "-I", os.path.join(ROOT, "include"),
                        "-o", str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    got = dict(l.split() for l in subprocess.run([str(exe)], capture_output=True,
                                                 text=True).stdout.splitlines())
    for name, cls in structs.items():
        assert int(got[name]) == ctypes.sizeof(cls), name
        for fname, _ in cls._fields_:
            assert int(got[f"{name}.{fname}"]) == getattr(cls, fname).offset, (name, fname)


def test_server_config_defaults():
    c = gg.gg_server_config()
    assert gg.LIB.gg_server_default_config(ctypes.byref(c)) == gg.OK
    assert c.streams == 2 and c.max_batch_jobs == 256 and c.hbm_budget_bytes == 150000000000
    assert c.options.mode == gg.MODE_WINDOW and c.options.accum == gg.ACC_COMPENSATED
    c.streams = 0
    h = ctypes.c_void_p()
    assert gg.LIB.gg_server_create(ctypes.byref(h), ctypes.byref(c)) == gg.ERR_ARG


def test_abi_version_and_defaults():
    assert gg.LIB.gg_abi_version() == 1
    o = gg.gg_options()
    assert gg.LIB.gg_default_options(ctypes.byref(o)) == gg.OK
    assert (o.mode, o.layout, o.accum, o.gcf_kind) == (
        gg.MODE_SCATTER, gg.LAYOUT_REFERENCE, gg.ACC_PLAIN, gg.GCF_TABLE)
    assert (o.oversample, o.polarizations, o.tile) == (8, 1, 0)


@pytest.mark.parametrize("field,value", [
    ("mode", 9), ("layout", 7), ("accum", 5), ("gcf_kind", 4),
    ("oversample", 6), ("oversample", 128), ("polarizations", 0),
    ("polarizations", 9), ("tile", 24), ("tile", 4), ("window_chunk", -1),
    ("autotune", 3), ("autotune", -1)])
def test_bad_options_rejected_with_message(field, value):
    o = gg.Options()
    c = o.c()
    setattr(c, field, value)
    assert gg.LIB.gg_set_global_options(ctypes.byref(c)) == gg.ERR_ARG
    assert field.split("_")[0] in gg.LIB.gg_last_error().decode()


def test_global_options_roundtrip():
    o = gg.Options(mode=gg.MODE_WINDOW, polarizations=4, oversample=16).c()
    assert gg.LIB.gg_set_global_options(ctypes.byref(o)) == gg.OK
    back = gg.gg_options()
    assert gg.LIB.gg_get_global_options(ctypes.byref(back)) == gg.OK
    assert (back.mode, back.polarizations, back.oversample) == (gg.MODE_WINDOW, 4, 16)
    gg.set_global_options(gg.Options())


def test_null_arguments_rejected():
    assert gg.LIB.gg_default_options(None) == gg.ERR_ARG
    assert gg.LIB.gg_grid_device(None, None, None, None) == gg.ERR_ARG
    assert gg.LIB.gg_degrid_device(None, None, None, None) == gg.ERR_ARG
    assert gg.LIB.gg_grid_to_image(None, None, 64, 1, gg.C64, None) == gg.ERR_ARG
    assert gg.LIB.gg_read_flags(None, None, None) == gg.ERR_ARG
    o = gg.Options().c()
    assert gg.LIB.gg_grid_host(ctypes.byref(o), 0, None, 0, None, 0, None, 1, 8,
                               None, 8) == gg.ERR_ARG


def test_context_without_gpu_fails_cleanly():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    h = ctypes.c_void_p()
    st = gg.LIB.gg_create(ctypes.byref(h), 0)
    assert st in (gg.ERR_CUDA, gg.ERR_NOMEM)
    assert gg.LIB.gg_last_error()


def test_padded_buffer_convention():
    # grid.cu:290 and grid_gpu.cu:732
    assert gg.padded_size(2048, 32) == 2048 * 2048 + 2 * 2048 * 32 + 64
    assert gg.grid_head(2048, 32) == 2048 * 32 + 32


def test_synthetic_generators():
    uv, v = synth.uniform(1000, 16, 1008, seed=1)
    assert uv.dtype == np.float64 and v.dtype == np.complex64
    assert np.array_equal(uv, uv.astype(np.float32).astype(np.float64))
    assert uv.min() >= 16 and uv.max() < 1008
    uv, v = synth.tracks(img_dim=512, nant=16, ntime=50, npts=16 * 15 // 2 * 50 + 7)
    assert uv.shape == (6007, 2)
    r = np.abs(uv - 256).max()
    assert 0.85 * 256 < r <= 0.9 * 256 + 1e-3
    uv, v = synth.disk(20000, 1024, outlier_frac=0.01, seed=2)
    assert (np.abs(v) > 100).sum() == 200
    rr = np.hypot(uv[:, 0] - 512, uv[:, 1] - 512)
    assert rr.max() <= 0.9 * 512 + 1e-3
    perm = synth.tile_sort(uv, 1024)
    m = np.clip(np.floor(uv[perm]).astype(int), 0, 1023)
    key = (m[:, 1] // 32) * 32 + m[:, 0] // 32
    assert np.all(np.diff(key) >= 0)


def test_gcf_table_matches_oracle_layout():
    import oracle as O
    g1 = synth.gaussian_gcf_1d(8)
    assert np.array_equal(synth.gcf_table(g1), O.gcf_from_1d(g1))


def test_header_constants_match_python_mirror():
    src = open(os.path.join(ROOT, "include", "gg.h")).read()
    consts = dict(re.findall(r"#define (GG_\w+) (-?\d+)", src))
    assert int(consts["GG_SERVER_TUNE_BATCHES"]) == gg.SERVER_TUNE_BATCHES
    assert int(consts["GG_REQ_KEEP_RESIDENT"]) == gg.REQ_KEEP_RESIDENT
    assert int(consts["GG_GCF_WPHASE"]) == gg.GCF_WPHASE


def test_noalloc_array_size_as_documented():
    """The size of the allocation-free entry point's fixed array stated in
    include/gg.h is the size of the array in libgg.so (symbol table)."""
    import shutil
    import subprocess
    nm = shutil.which("nm")
    if not nm:
        pytest.skip("no nm")
    hdr = open(os.path.join(ROOT, "include", "gg.h")).read()
    m = re.search(r"array \((\d+) bytes", hdr)
    assert m, "gg.h states the array size in bytes"
    out = subprocess.run([nm, "-S", "-C", gg.LIB_PATH], capture_output=True, text=True).stdout
    sizes = [int(line.split()[1], 16) for line in out.splitlines()
             if "g_noalloc_scratch" in line and len(line.split()) >= 4]
    assert sizes == [int(m.group(1))], sizes
