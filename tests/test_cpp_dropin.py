"""The C-ABI boundary exercised from C and C++ rather than ctypes.

tests/cpp/dropin_main.cpp is the reference's main() (src/spgemm_raw_v2.cu:61-
243) rewritten against include/spgemm_gb300.h: tile A and B, run steps 1-3,
print the reference's timing line, read C back.  The CPU tests compile it with
g++ (and the header alone as C99 with gcc) and link it to libspgemm_gb300.so;
the GPU tests run it and compare C with the CPU oracle bit for bit (structure)
and within the value tolerance."""
import os
import subprocess

import numpy as np
import pytest

import oracle
from gpu_spgemm_gb300 import build as lib_build
from gpu_spgemm_gb300 import synth

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "dropin_main.cpp")
INC = os.path.join(ROOT, "include")
LIBDIR = os.path.dirname(lib_build.LIB)
STRUCT_KEYS = ["tile_ptrC", "tile_rowidxC", "tile_colidxC", "maskC", "tile_nnzC", "ptrRowC", "tile_colC"]


def compile_dropin(out_dir) -> str:
    lib_build.build()
    exe = os.path.join(str(out_dir), "dropin_main")
    subprocess.run(["g++", "-O2", "-std=c++17", "-Wall", "-Wextra", "-Werror", "-I", INC, SRC, "-L", LIBDIR,
                    "-lspgemm_gb300", "-Wl,-rpath," + LIBDIR, "-o", exe], check=True, capture_output=True, text=True)
    return exe


def test_header_is_valid_c99(tmp_path):
    c = tmp_path / "use_header.c"
    c.write_text('#include "spgemm_gb300.h"\n'
                 'int main(void) { spg_handle_t h = 0; spg_stats st; (void)h; (void)st;\n'
                 '  return (int)sizeof(spg_tiles) > 0 ? 0 : 1; }\n')
    subprocess.run(["gcc", "-std=c99", "-Wall", "-Wextra", "-pedantic", "-Werror", "-I", INC, "-c", str(c),
                    "-o", str(tmp_path / "use_header.o")], check=True, capture_output=True, text=True)


def test_dropin_compiles_and_links(tmp_path):
    exe = compile_dropin(tmp_path)
    assert os.access(exe, os.X_OK)


def write_csr(path, a):
    dt = 1 if a.val.dtype == np.float64 else 0
    with open(path, "wb") as f:
        np.array([a.m, a.n], np.int32).tofile(f)
        np.array([a.nnz], np.int64).tofile(f)
        np.array([dt], np.int32).tofile(f)
        np.ascontiguousarray(a.row_ptr, np.int32).tofile(f)
        np.ascontiguousarray(a.col_idx, np.int32).tofile(f)
        np.ascontiguousarray(a.val).tofile(f)


def read_c(path, dtype):
    with open(path, "rb") as f:
        nt, nz, tilem = np.fromfile(f, np.int64, 3)
        out = dict(numtileC=int(nt), nnzC=int(nz))
        for k, t, n in (("tile_ptrC", np.int32, tilem + 1), ("tile_rowidxC", np.int32, nt),
                        ("tile_colidxC", np.int32, nt), ("maskC", np.uint16, nt * 16), ("tile_nnzC", np.int64, nt + 1),
                        ("ptrRowC", np.uint8, nt * 16), ("tile_colC", np.uint8, nz), ("tile_valC", dtype, nz)):
            out[k] = np.fromfile(f, t, int(n))
    return out


@pytest.mark.gpu
@pytest.mark.parametrize("name,a,algo", [("poisson2d_64_f64", synth.poisson2d(64), "auto"),
                                         ("rmat_11_f32", synth.rmat(11, 16), "rowwise"),
                                         ("stencil27_4_f32", synth.stencil27_dof3(4), "plain")])
def test_dropin_runs_and_matches_oracle(tmp_path, name, a, algo):
    exe = compile_dropin(tmp_path)
    fin, fout = tmp_path / "in.bin", tmp_path / "out.bin"
    write_csr(fin, a)
    r = subprocess.run([exe, str(fin), str(fout), algo], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert "GFlops" in r.stdout
    got = read_c(fout, a.val.dtype)
    S = oracle.spgemm_tiles(a, a)
    assert got["numtileC"] == S["numtileC"] and got["nnzC"] == S["nnzC"]
    for k in STRUCT_KEYS:
        np.testing.assert_array_equal(got[k], S[k].astype(got[k].dtype), err_msg=k)
    ref = S["tile_valC"]
    err = np.linalg.norm(got["tile_valC"].astype(np.float64) - ref) / np.linalg.norm(ref)
    assert err <= (1e-12 if a.val.dtype == np.float64 else 1e-6), err
