"""The OCaml C stubs (mmo_gb300/ocaml/mmo_gpu_stubs.c) compile against the C
ABI.  There is no OCaml toolchain here, so tests/ocaml_shim stands in for the
OCaml runtime headers; this checks the stubs' C and their use of the ABI."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.skipif(shutil.which("gcc") is None, reason="gcc missing")
def test_ocaml_stub_compiles_against_abi(tmp_path):
    out = tmp_path / "stubs.o"
    r = subprocess.run(["gcc", "-c", "-Wall", "-Wextra", "-Werror", "-std=c99", "-fPIC",
                        "-I", os.path.join(ROOT, "tests", "ocaml_shim"),
                        "-I", os.path.join(ROOT, "include"),
                        os.path.join(ROOT, "mmo_gb300", "ocaml", "mmo_gpu_stubs.c"),
                        "-o", str(out)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    syms = subprocess.run(["nm", str(out)], capture_output=True, text=True).stdout
    for name in ("mmo_ocaml_create", "mmo_ocaml_set_protein", "mmo_ocaml_set_ligand_byte",
                 "mmo_ocaml_ene_inter", "mmo_ocaml_ene_intra", "mmo_ocaml_score_poses",
                 "mmo_ocaml_score_config", "mmo_ocaml_build_grids", "mmo_ocaml_ene_inter_grid"):
        assert " T " + name in syms, name
    # every ABI call the stubs make is a symbol the library exports
    for call in ("mmo_ctx_create", "mmo_set_ligand", "mmo_ene_inter", "mmo_score_poses",
                 "mmo_build_grids", "mmo_ene_inter_grid"):
        assert " U " + call in syms


def test_ml_externals_match_stub_symbols():
    ml = open(os.path.join(ROOT, "mmo_gb300", "ocaml", "ff_gpu.ml")).read()
    c = open(os.path.join(ROOT, "mmo_gb300", "ocaml", "mmo_gpu_stubs.c")).read()
    import re

    for name in re.findall(r'"(mmo_ocaml_[a-z_]+)"', ml):
        assert "CAMLprim value " + name + "(" in c, name
