"""decompose.py end to end on the GPU, as a user runs it: the output JSON has
the reference's keys (decompose.py:117-137) and its statistics the keys and
nesting of ALS_Optimizer::get_statistics_json (als_optimizer.hpp:99-123,
captured from the reference in tests/golden/stats_*.json); trials resume as
the reference's do (decompose.py:188-214); factors written with
--factor-file restart a run with --init-factors."""
import json
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

# The reference's output dictionary (decompose.py:117-137); this build adds "precision".
REFERENCE_KEYS = {"time", "metadata", "input", "target_rank", "iterations", "algorithm", "preprocessing",
                  "data_distribution", "sample_count", "accuracy_epoch_length", "trial_count", "trial_num",
                  "initial_fit", "final_fit", "thread_count", "node_count", "mpi_rank_count", "stats"}


def run(args, timeout=600):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "decompose.py"), *args], cwd=ROOT, capture_output=True,
                       text=True, timeout=timeout)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    return r.stdout


@pytest.mark.parametrize("alg", ["sts_cp", "cp_arls_lev"])
def test_decompose_output_schema_and_trial_resume(tmp_path, alg):
    out = tmp_path / "out"
    out.mkdir()
    args = ["-i", "synthetic:planted", "-t", "8", "-iter", "3", "-alg", alg, "-s", "8192", "-dist",
            "accumulator_stationary", "-e", "1", "-o", str(out), "-r", "2", "-m", "t"]
    run(args)
    files = sorted(os.listdir(out))
    assert len(files) == 1 and files[0].endswith("_0.out"), files
    d = json.load(open(out / files[0]))
    assert set(d) == REFERENCE_KEYS | {"precision"}
    assert d["trial_num"] == 0 and d["target_rank"] == 8 and d["algorithm"] == alg and d["mpi_rank_count"] == 1
    with open(os.path.join(ROOT, "tests", "golden", f"stats_{alg}.json")) as f:
        ref = json.load(f)
    st = d["stats"]
    assert set(st) == set(ref)
    for k, v in ref.items():
        if isinstance(v, dict):
            assert set(st[k]) == set(v), k
    assert st["rounds"] == [0, 1, 2, 3] and len(st["fits"]) == 4
    assert st["fits"][-1] == pytest.approx(d["final_fit"], abs=1e-12)
    # the second invocation runs trial 1, the third finds nothing left to do
    run(args)
    assert sorted(os.listdir(out))[1].endswith("_1.out")
    assert "No trials left to perform!" in run(args)


def test_decompose_exact_preprocessing_and_factor_resume(tmp_path):
    ff = str(tmp_path / "factors.npz")
    common = ["-i", "synthetic:planted", "-t", "6", "-alg", "sts_cp", "-s", "8192", "-dist",
              "tensor_stationary", "-e", "1"]
    text = run(common + ["-iter", "2", "-p", "exact", "--factor-file", ff])
    assert "Executing single round of Exact ALS as preprocessing..." in text
    assert os.path.exists(ff)
    first = json.loads(text[text.index("{"): text.rindex("}") + 1])
    text2 = run(common + ["-iter", "1", "--init-factors", ff])
    second = json.loads(text2[text2.index("{"): text2.rindex("}") + 1])
    # the resumed run starts from the fit the first one ended with
    assert second["initial_fit"] == pytest.approx(first["final_fit"], abs=1e-12)
