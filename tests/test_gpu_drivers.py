"""The reference's driver CLI over libamps (w3914777_gb300/drivers/amps_driver.cpp):
snowflake/purehigh.cu, graingrowth/end2end_mix.cu, snowflake/purelow.cu and
sintering/main.cu calling conventions and outputs (time_tmp.csv, the CSV
dump format of snowflake/tools.h:4-23, the sintering result tree)."""
import os
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB = os.path.join(ROOT, "w3914777_gb300", "_lib")
GOLD = os.path.join(ROOT, "tests", "golden")


def run(prog, *args, cwd):
    r = subprocess.run([os.path.join(LIB, prog), *args], cwd=cwd, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    return r


def read_csv(path):
    with open(path) as f:
        head = f.readline().strip().split(",")
        rows = [line.strip().split(",") for line in f]
    assert head[0] == "" and head[1:] == [str(i) for i in range(len(head) - 1)]
    assert [int(r[0]) for r in rows] == list(range(len(rows)))
    return np.array([[float(v) for v in r[1:]] for r in rows])


def test_snowflake_purehigh_cli_dumps_the_reference_field(tmp_path):
    g = np.load(os.path.join(GOLD, "kobayashi_ref.npz"))
    run("snowflake_purehigh", "4", "phi.csv", "--para", "2", "--timesteps", str(int(g["early"])), cwd=tmp_path)
    phi = read_csv(tmp_path / "phi.csv")
    # 6 significant digits: the reference's default ostream formatting
    assert np.allclose(phi, g["phi_early"], rtol=1e-5, atol=1e-6)
    assert float(open(tmp_path / "time_tmp.csv").read()) > 0


def test_graingrowth_end2end_mix_cli(tmp_path):
    run("graingrowth_end2end_mix", "4", "eta2.csv", "--para", "1", "--timesteps", "40", "--threshold", "1e-4",
        cwd=tmp_path)
    eta2 = read_csv(tmp_path / "eta2.csv")
    g = np.load(os.path.join(GOLD, "graingrowth_ref.npz"))
    assert np.max(np.abs(eta2 - g["eta2"])) < 5e-3


def test_purelow_cli_writes_half2result(tmp_path):
    out = run("snowflake_purelow", "--timesteps", "20", cwd=tmp_path).stdout
    assert "half2result.csv" in out
    assert read_csv(tmp_path / "half2result.csv").shape == (512, 512)


def test_sintering_main_cli_result_tree(tmp_path):
    g = np.load(os.path.join(GOLD, "sintering_ref.npz"))
    run("sintering_main", "5", "double", "--timesteps", str(int(g["steps"])), cwd=tmp_path)
    c = read_csv(tmp_path / "result" / "end2end" / "double" / "pure" / "para5" / f"{int(g['steps'])}.csv")
    assert np.allclose(c, g["c"], rtol=1e-5, atol=1e-6)
    run("sintering_main", "5", "double", "--timesteps", "20", "--strategy", "amstencil", "--threshold", "0.001",
        cwd=tmp_path)
    assert (tmp_path / "result" / "end2end" / "double" / "amstencil" / "monitor2" / "para5" / "20_0.001.csv").exists()
