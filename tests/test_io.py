"""Configuration and result files (common/ConfigParser.cpp, common/Loader.cpp,
common/Results.cpp) through the C ABI, against the reference's own outputs
in tests/golden/ (no GPU needed)."""
import json
import os

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(__file__), "golden")
CFG = os.path.join(GOLD, "configs")


@pytest.mark.parametrize("name", ["plain", "comments_case_blanks", "duplicate_first_wins",
                                  "single_char_value_kept_blanks", "triple_slash_comment",
                                  "blank_only_value", "last_line_without_newline"])
def test_read_config_matches_reference(eng, name):
    exp = json.load(open(os.path.join(CFG, "expected.json")))[name]
    cfg, strings, extra = eng.read_config(os.path.join(CFG, name + ".cfg"))
    ints, floats, strs = exp["ints"], exp["floats"], exp["strings"]
    assert [cfg.n_lj, cfg.n_mb, cfg.timesteps, int(extra["CUDA Blocks"]), cfg.output_timesteps,
            int(extra["AnimationTimesteps"])] == ints[:6]
    assert [cfg.use_lj, cfg.use_mb] == ints[7:9]
    got_f = [cfg.dt, extra["Temperature"], cfg.lj_rs, cfg.lj_rcut, cfg.mb_rs, cfg.mb_rcut,
             extra["VXCMFROM"], extra["VXCMTO"], extra["VXCMSTEP"], cfg.energy_loss]
    assert np.array_equal(np.float32(got_f), np.float32(floats))
    assert [strings[k] for k in ("Input", "Output", "Filename", "AnimationData")] == strs
    # extension keys absent: the reference's behaviour
    assert (cfg.periodic, cfg.precision, cfg.species) == (0, 0, 0)


@pytest.mark.parametrize("name", ["bad_missing_key", "bad_no_equals", "bad_key_with_blank"])
def test_bad_config_is_an_error_not_an_exit(eng, name):
    with pytest.raises(eng.EngineError) as ei:
        eng.read_config(os.path.join(CFG, name + ".cfg"))
    assert ei.value.status == 1  # MD_BAD_CONFIG


def test_bad_line_names_the_key_lines_before_it(eng, tmp_path):
    """ConfigParser.cpp:60-64: the line number in the message counts the
    key lines read so far; comments and empty lines do not count."""
    p = tmp_path / "c.cfg"
    p.write_text("// c\n\nA=1\n\n// d\nB=2\nno equals here\n")
    with pytest.raises(eng.EngineError) as ei:
        eng.read_config(str(p))
    assert "Line: 2" in str(ei.value)
    p.write_text("A=1\n=2\n")
    with pytest.raises(eng.EngineError) as ei:
        eng.read_config(str(p))
    assert "Line: 1" in str(ei.value)


def test_extension_keys(eng, tmp_path):
    text = open(os.path.join(CFG, "plain.cfg")).read()
    p = tmp_path / "ext.cfg"
    p.write_text(text + "Periodic=1\nBox=34.31\nPrecision=mixed\nSpecies=argon\n")
    cfg, _, _ = eng.read_config(str(p))
    assert (cfg.periodic, cfg.precision, cfg.species) == (1, 1, 1)
    assert abs(cfg.box - 34.31) < 1e-12
    p.write_text(text + "Precision=fp16\n")
    with pytest.raises(eng.EngineError):
        eng.read_config(str(p))


def test_results_files_are_byte_identical(eng, tmp_path):
    """writeResults + tailResults (common/Results.cpp:88-229)."""
    import ctypes as C
    recs = np.load(os.path.join(GOLD, "results_records.npy"))
    gold = np.load(os.path.join(GOLD, "reference_fixtures.npz"))
    pos = np.ascontiguousarray(gold["bo_no/pos"])
    cfg = eng.make_config(n_lj=0, n_mb=len(pos), dt=2.0, timesteps=200, lj_rs=9.0, lj_rcut=8.0,
                          use_lj=0, use_mb=1, mb_rs=3.5, mb_rcut=3.0)
    th = np.zeros((3, 16))
    th[:, :11] = recs
    th = np.ascontiguousarray(th)
    stem = str(tmp_path / "res")
    L = eng.load()
    s = L.md_write_results(stem.encode(), C.byref(cfg), 0.5, 123.0, th.ctypes.data, 3,
                           pos.ctypes.data)
    assert s == 0
    for ext in ("dat", "txt"):
        mine = open(f"{stem}(vxcm-0.5).{ext}", "rb").read()
        ref = open(os.path.join(GOLD, f"results_vxcm-0.5.{ext}"), "rb").read()
        assert mine == ref, ext


def test_results_files_from_a_pair_list(eng, tmp_path):
    """md_write_results_pairs (the pair list given, as md_tail_pairs returns
    it) writes the same bytes as the reference's writeResults."""
    import ctypes as C
    recs = np.load(os.path.join(GOLD, "results_records.npy"))
    gold = np.load(os.path.join(GOLD, "reference_fixtures.npz"))
    pos = np.ascontiguousarray(gold["bo_no/pos"])
    n = len(pos)
    cfg = eng.make_config(n_lj=0, n_mb=n, dt=2.0, timesteps=200, lj_rs=9.0, lj_rcut=8.0,
                          use_lj=0, use_mb=1, mb_rs=3.5, mb_rcut=3.0)
    # tailResults restated (common/Results.cpp:88-118)
    lim = float(np.float32(2) * np.float32(1.15))
    pairs = []
    for i in range(n):
        for j in range(i + 1, n):
            if int(pos[i, 3]) == int(pos[j, 3]):
                continue
            dx, dy, dz = pos[i, :3] - pos[j, :3]
            if np.sqrt(dx * dx + dy * dy + dz * dz) < lim:
                pairs += [i, j]
    flat = np.ascontiguousarray(np.array(pairs, np.int32))
    th = np.zeros((3, 16))
    th[:, :11] = recs
    th = np.ascontiguousarray(th)
    stem = str(tmp_path / "res")
    L = eng.load()
    s = L.md_write_results_pairs(stem.encode(), C.byref(cfg), 0.5, 123.0, th.ctypes.data, 3,
                                 flat.ctypes.data, len(flat) // 2)
    assert s == 0
    for ext in ("dat", "txt"):
        mine = open(f"{stem}(vxcm-0.5).{ext}", "rb").read()
        ref = open(os.path.join(GOLD, f"results_vxcm-0.5.{ext}"), "rb").read()
        assert mine == ref, ext


def test_input_output_text_format(tmp_path, reference):
    """lattice.write_input writes what the reference's readInput reads."""
    from moleculardynamics_gb300 import lattice as lat
    pos, vel, _ = lat.make_system("fcc", 2, 94.4, seed=3)
    path = str(tmp_path / "input.txt")
    lat.write_input(path, pos, vel)
    p2 = np.zeros_like(pos)
    v2 = np.zeros_like(vel)
    reference.lib.ref_read_input(path.encode(), len(pos), p2, v2)
    a, b = lat.read_input(path, len(pos))
    assert np.array_equal(a, p2) and np.array_equal(b, v2)
    assert np.allclose(p2, pos, rtol=1e-6) and np.allclose(v2, vel, rtol=1e-6)
