"""The generator's command line writes the drop-in pair for a program."""
import os
import subprocess
import sys

from formura_gb300 import build as B

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_cli_generates_compilable_pair(tmp_path):
    src, _ = B.program_sources("gs2d")
    (tmp_path / "gs2d.fmr").write_text(src)
    (tmp_path / "gs2d.yaml").write_text("length_per_node: [1.28, 1.28]\ngrid_per_node: [128, 128]\n")
    env = dict(os.environ, PYTHONPATH=ROOT)
    r = subprocess.run([sys.executable, "-m", "formura_gb300.generator.cli", "-v", str(tmp_path / "gs2d.fmr")],
                       capture_output=True, text=True, env=env)
    assert r.returncode == 0, r.stderr
    assert "sleeve: 1" in r.stdout and "Generate:" in r.stdout
    h = (tmp_path / "gs2d.h").read_text()
    for sym in ("Formura_Grid_Struct", "Formura_Navi", "to_pos_x", "Formura_Init", "Formura_Forward",
                "Formura_Finalize", "double u[128][128];"):
        assert sym in h
    r = subprocess.run(["gcc", "-c", "-std=c11", "-I", os.path.join(ROOT, "include"), str(tmp_path / "gs2d.c"),
                        "-o", str(tmp_path / "gs2d.o")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_cli_reports_config_errors(tmp_path):
    (tmp_path / "p.fmr").write_text("dimension :: 1\naxes :: x\n")
    (tmp_path / "p.yaml").write_text("length_per_node: [1.0]\n")
    env = dict(os.environ, PYTHONPATH=ROOT)
    r = subprocess.run([sys.executable, "-m", "formura_gb300.generator.cli", str(tmp_path / "p.fmr")],
                       capture_output=True, text=True, env=env)
    assert r.returncode == 1 and "grid_per_node" in r.stderr
