"""The C-ABI library: loads, exports every function include/*.h declares, and
keeps its struct layouts (no compute on the GPU here)."""
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INCLUDE = os.path.join(ROOT, "include")


def declared_functions():
    names = set()
    for f in os.listdir(INCLUDE):
        if f.endswith(".h"):
            text = open(os.path.join(INCLUDE, f)).read()
            text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
            for m in re.finditer(r"\b((?:md|mdgb)_[a-z0-9_]+)\s*\(", text):
                names.add(m.group(1))
    return sorted(names)


def test_every_declared_function_is_exported(eng):
    lib = eng.load()
    names = declared_functions()
    assert len(names) >= 30
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    assert sorted(eng.EXPORTS) == names


def test_struct_layouts_match_the_header(eng, tmp_path):
    import ctypes as C
    src = tmp_path / "sz.c"
    src.write_text('#include "mdgb.h"\n#include <stdio.h>\n#include <stddef.h>\n'
                   'int main(void){printf("%zu %zu %zu %zu %zu %zu\\n", sizeof(md_config),'
                   ' sizeof(md_thermo), sizeof(md_stats), sizeof(mdgb_list_settings),'
                   ' sizeof(md_tune_result), sizeof(md_surrogate_stats));return 0;}\n')
    exe = tmp_path / "sz"
    subprocess.run(["gcc", "-I", INCLUDE, str(src), "-o", str(exe)], check=True)
    sizes = [int(x) for x in subprocess.run([str(exe)], capture_output=True, text=True,
                                            check=True).stdout.split()]
    assert sizes == [C.sizeof(eng.MdConfig), C.sizeof(eng.MdThermo), C.sizeof(eng.MdStats),
                     C.sizeof(eng.ListSettings), C.sizeof(eng.MdTuneResult),
                     C.sizeof(eng.MdSurrogateStats)]
    assert C.sizeof(eng.MdThermo) == 16 * 8


def test_status_strings(eng):
    lib = eng.load()
    for s in range(10):
        assert lib.md_status_string(s)


def test_create_without_a_device_fails_cleanly(eng):
    """No CUDA device here: md_create returns MD_NO_DEVICE, nothing exits."""
    import ctypes as C
    lib = eng.load()
    n = C.c_int()
    cudart = None
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    h = C.c_void_p()
    cfg = eng.make_config(n_lj=8)
    assert lib.md_create(C.byref(cfg), C.byref(h)) == 7
    bad = eng.make_config(n_lj=0, n_mb=0)
    assert lib.md_create(C.byref(bad), C.byref(h)) == 1  # MD_BAD_CONFIG before the device


def test_bad_configs_are_rejected(eng):
    import ctypes as C
    lib = eng.load()
    h = C.c_void_p()
    for cfg in (eng.make_config(n_lj=10, lj_rs=8.0, lj_rcut=9.0),
                eng.make_config(n_lj=10, dt=0.0),
                eng.make_config(n_lj=10, periodic=1, box=10.0),
                eng.make_config(n_lj=10, precision=7),
                eng.make_config(n_mb=10, use_lj=0, use_mb=1, mb_rs=3.0, mb_rcut=3.5),
                eng.make_config(n_lj=10, cluster_stage_cap=32),
                eng.make_config(n_lj=10, cluster_stage_cap=20000)):
        assert lib.md_create(C.byref(cfg), C.byref(h)) == 1


def test_library_links_only_cuda_runtime(eng):
    out = subprocess.run(["ldd", eng.LIB_PATH], capture_output=True, text=True).stdout
    assert "libcudart" in out or "cudart" in out
    assert "torch" not in out and "python" not in out


def test_surrogate_model_calls_reject_bad_arguments(eng):
    """The head, scale and range entry points check their arguments before
    touching a device: a NULL surrogate or NULL arrays are MD_BAD_ARGUMENT."""
    import ctypes as C
    import numpy as np
    lib = eng.load()
    assert [lib.md_surrogate_head_param_count(h) for h in (32, 64, 128)] == [
        h * 32 + h + h * h + h + 32 * h + 32 for h in (32, 64, 128)]
    assert lib.md_surrogate_head_param_count(48) == -1
    p = np.zeros(8, np.float32)
    assert lib.md_surrogate_set_model(None, 1, 64) == 6
    assert lib.md_surrogate_head_params(None, p, 8, 0) == 6
    d = C.c_double(1.0)
    assert lib.md_surrogate_head_scale(None, C.byref(d), 1) == 6
    lo, hi = np.zeros(32, np.float32), np.ones(32, np.float32)
    assert lib.md_surrogate_range(None, lo, hi, 1) == 6
    x = np.zeros(32, np.float32)
    assert lib.md_surrogate_head_grad(None, x, x, 1, p) == 6
