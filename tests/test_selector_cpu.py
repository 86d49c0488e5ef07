"""Selector host logic without a GPU: feature map, threshold rule, model
persistence and the checks gb_selector_load_file makes before any device
work (magic, version, size, CRC-32)."""
import json
import os

import numpy as np
import pytest

from blis_gb300 import _lib
from blis_gb300 import selector as S

TUNING = os.path.join(os.path.dirname(__file__), "..", "blis_gb300", "tuning")


def test_features_and_rule():
    f = S.features(300, 20, 4000, 0, 1, 0, 8, 10.0, 0.0)
    assert f.shape == (S.NIN,) and f.dtype == np.float32
    assert f[3] == 1 and f[6] == 1 and f[9] == 1 and f[15] == 1
    assert S.heuristic_config(300, 300, 300) == 0
    assert S.heuristic_config(6, 800, 800) == 1


def test_sampled_shapes_respect_caps():
    shapes = S.sample_shapes(500, seed=9)
    for sh in shapes:
        assert 2.0 * sh["m"] * sh["n"] * sh["k"] <= S.WORK_CAP
        assert max(sh["m"] * sh["k"], sh["k"] * sh["n"], sh["m"] * sh["n"]) <= S.ELEM_CAP
        assert sh["pad"] in S.PADS


def test_committed_model_and_evaluation():
    p, doc = S.load_model(os.path.join(TUNING, "selector_mlp.json"))
    assert p.size == S.NPARAMS and doc["meta"]["train_samples"] == 20000
    ev = json.load(open(os.path.join(TUNING, "selector_eval_heldout.json")))
    assert ev["n"] == 2000
    assert ev["mlp"]["mean_throughput_regret"] <= 0.05
    assert ev["mlp"]["mean_throughput_regret"] < ev["threshold_rule"]["mean_throughput_regret"]
    # measured: the Ozaki form run at every final slice count, errors in double-double
    meas = ev["slices"]["measured"]
    assert meas["shapes"] == ev["slices"]["n"] and meas["bound_violations"] == 0
    assert ev["slices"]["violations_after_verifier"] == 0
    train = [np.load(os.path.join(TUNING, f)) for f in ("autotune_train.npz", "autotune_train2.npz")]
    assert sum(t["X"].shape[0] for t in train) == 20000
    raw = open(os.path.join(TUNING, "selector_mlp.bin"), "rb").read()
    assert raw[:8] == S.BIN_MAGIC and np.array_equal(np.frombuffer(raw[20:], "<f4"), p)


def test_load_file_rejects_corrupt_models(gblib, tmp_path):
    p, _ = S.load_model(os.path.join(TUNING, "selector_mlp.json"))
    good = tmp_path / "good.bin"
    S.save_model_bin(str(good), p)
    raw = bytearray(good.read_bytes())
    raw[100] ^= 0x40  # flip a parameter bit: CRC mismatch
    bad = tmp_path / "bad.bin"
    bad.write_bytes(bytes(raw))
    assert gblib.gb_selector_load_file(str(bad).encode()) != 0
    trunc = tmp_path / "trunc.bin"
    trunc.write_bytes(bytes(raw[:1000]))
    assert gblib.gb_selector_load_file(str(trunc).encode()) != 0
    assert gblib.gb_selector_load_file(str(tmp_path / "missing.bin").encode()) != 0
    gblib.gb_clear_last_error()
    with pytest.raises(ValueError):
        doc = json.load(open(os.path.join(TUNING, "selector_mlp.json")))
        doc["params"][0] += 1.0
        path = tmp_path / "m.json"
        path.write_text(json.dumps(doc))
        S.load_model(str(path))
    code, _ = _lib.last_error()
    assert code == 0


def test_committed_model_regret_per_dtype_on_cpu():
    """The committed model's choices on the held-out shapes, recomputed with the
    FP64 restatement of the network: below 5% mean throughput regret for every
    dtype and better than the threshold rule."""
    from oracle import mlp_ref as R
    p, _ = S.load_model(os.path.join(TUNING, "selector_mlp.json"))
    d = np.load(os.path.join(TUNING, "autotune_heldout.npz"))
    pred = R.forward(p.astype(np.float64), d["X"].astype(np.float64))
    T, sh = d["T"], d["shapes"]
    best = T.min(1)
    t_mlp = T[np.arange(len(T)), pred[:, :S.NCONFIG].argmin(1)]
    rule = np.array([S.heuristic_config(int(r[0]), int(r[1]), int(r[2])) for r in sh])
    t_rule = T[np.arange(len(T)), rule]
    for code in (0, 1, 2):
        sel = sh[:, 3] == code
        assert sel.sum() >= 600
        regret = 1.0 - np.mean(best[sel] / t_mlp[sel])
        assert regret < 0.05 and regret < 1.0 - np.mean(best[sel] / t_rule[sel])


def test_occupancy_rule_between_threshold_rule_and_model():
    """Without a model the library uses the occupancy rule; on the held-out FP64 and FP32
    shapes it is better than BLIS's threshold rule and worse than the trained model."""
    from oracle import mlp_ref as R
    p, _ = S.load_model(os.path.join(TUNING, "selector_mlp.json"))
    d = np.load(os.path.join(TUNING, "autotune_heldout.npz"))
    pred = R.forward(p.astype(np.float64), d["X"].astype(np.float64))
    T, sh = d["T"], d["shapes"]
    best = T.min(1)
    idx = np.arange(len(T))
    t_mlp = T[idx, pred[:, :S.NCONFIG].argmin(1)]
    t_occ = T[idx, [S.occupancy_config(int(r[0]), int(r[1]), int(r[2])) for r in sh]]
    t_thr = T[idx, [S.heuristic_config(int(r[0]), int(r[1]), int(r[2])) for r in sh]]
    for code in (0, 1):
        sel = sh[:, 3] == code
        r_mlp, r_occ, r_thr = (float(np.mean(t[sel] / best[sel])) - 1.0 for t in (t_mlp, t_occ, t_thr))
        assert r_mlp < r_occ < r_thr, (code, r_mlp, r_occ, r_thr)


def test_engine_output_beats_rules_on_heldout():
    """The Ozaki engine output (CTA pairs or single CTAs per shape) of the committed model,
    recomputed on the CPU: on the engine-tuned held-out FP64 shapes its mean time over the
    exhaustive best is below always-pairs, always-single-CTA and the library's size rule."""
    from oracle import mlp_ref as R
    p, doc = S.load_model(os.path.join(TUNING, "selector_mlp.json"))
    assert doc["meta"].get("engine_output")
    raw = open(os.path.join(TUNING, "selector_mlp.bin"), "rb").read()
    assert int(np.frombuffer(raw[8:12], "<u4")[0]) == 2  # file version 2: the engine output is trained
    d = np.load(os.path.join(TUNING, "autotune_heldout.npz"))
    TE, sh = d["TE"], d["shapes"]
    tuned = TE[:, 1] > 0
    assert tuned.sum() >= 600
    pred = R.forward(p.astype(np.float64), d["X"][tuned].astype(np.float64))
    te = TE[tuned]
    best = te.min(1)
    rows = np.arange(len(te))
    t_mlp = te[rows, np.where(pred[:, S.OUT_ENGINE] >= 0.0, 1, 0)]
    t_rule = te[rows, [S.ozaki_engine_rule(int(r[0]), int(r[1]), int(r[2])) - 1 for r in sh[tuned]]]
    r_mlp, r_rule = np.mean(t_mlp / best), np.mean(t_rule / best)
    r_pair, r_one = np.mean(te[:, 1] / best), np.mean(te[:, 0] / best)
    assert r_mlp < r_rule < r_pair and r_mlp < r_one, (r_mlp, r_rule, r_pair, r_one)
    ev = json.load(open(os.path.join(TUNING, "selector_eval_heldout.json")))
    assert abs(ev["ozaki_engine"]["mlp_mean_time_over_best"] - r_mlp) < 1e-3
