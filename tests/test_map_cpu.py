"""Invariants of the constant STV -> 384 maps (kqed_stv_map.h) that the
float assembly relies on, checked without a GPU: coefficients are +-1/2,
+-1, +-2 (the table of scaled copies has one slot per code), the +-1/2
terms use columns 0..7 only (the table's span), and the round lengths of
the warp schedule (rows sorted by length, dealt 32 per round) equal the
compile-time constants map_round_len of kqed_internal.h."""
import os
import re
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "kqed_gb300", "csrc")


def _arrays(name):
    src = open(os.path.join(CSRC, "kqed_stv_map.h")).read()
    out = {}
    for part in ("ROW", "COL", "Q4"):
        body = re.search(r"KQ_MAP_%s_%s\[\d+\] = \{(.*?)\};" % (name, part), src, re.S).group(1)
        out[part] = [int(v) for v in body.replace("\n", "").split(",") if v.strip()]
    return out


def _round_lengths(row):
    nnz = [row[i + 1] - row[i] for i in range(384)]
    order = sorted(range(384), key=lambda i: -nnz[i])     # stable, as std::stable_sort
    return [max(nnz[order[r * 32 + l]] for l in range(32)) for r in range(12)]


@pytest.mark.parametrize("name", ["GEN", "ZERO"])
def test_map_coefficients_and_columns(name):
    m = _arrays(name)
    assert len(m["ROW"]) == 385 and m["ROW"][0] == 0 and m["ROW"][-1] == len(m["COL"])
    assert set(m["Q4"]) <= {-8, -4, -2, 2, 4, 8}
    for c, q in zip(m["COL"], m["Q4"]):
        assert 0 <= c < 200
        if abs(q) == 2:
            assert c < 8                  # the 1/2 copies hold columns 0..7 only


def test_round_lengths_match_the_compiled_constants(tmp_path):
    gxx = shutil.which("g++")
    cuda_inc = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "include")
    if not gxx or not os.path.exists(os.path.join(cuda_inc, "cuda_runtime.h")):
        pytest.skip("g++ or the CUDA headers are not available")
    prog = tmp_path / "len.cpp"
    prog.write_text('#include "kqed_internal.h"\n#include <cstdio>\n'
                    "int main() { for (int g = 1; g >= 0; g--) { for (int r = 0; r < kqed::kMapRounds; r++)"
                    ' printf("%d ", kqed::map_round_len(g, r)); printf("\\n"); } }\n')
    exe = str(tmp_path / "len")
    subprocess.run([gxx, "-std=c++17", "-I", CSRC, "-I", cuda_inc, str(prog), "-o", exe],
                   check=True, capture_output=True)
    lines = subprocess.run([exe], check=True, capture_output=True, text=True).stdout.split("\n")
    compiled = [[int(v) for v in ln.split()] for ln in lines[:2]]
    assert compiled[0] == _round_lengths(_arrays("GEN")["ROW"])
    assert compiled[1] == _round_lengths(_arrays("ZERO")["ROW"])
