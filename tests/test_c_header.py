"""The C ABI is usable from plain C: include/pwa_gb300.h compiles as C99 and
C++17, and a C program linked against libpwa_gb300.so runs the host-side
setup of a likelihood (wave list and parameter layout, pwaLikelihood.cc:
1445-1556) and reads the error message of a refused call, with no GPU."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INC = os.path.join(ROOT, "include")
LIBDIR = os.path.join(ROOT, "rootpwa_gb300")

PROGRAM = r"""
#include <stdio.h>
#include <string.h>
#include "pwa_gb300.h"

int main(void)
{
    pwa_likelihood* L = 0;
    const char* names[3] = {"1-(1++)0+ rho pi S", "1-(2++)1+ rho pi D", "1-(0-+)0+ f0 pi S"};
    const int32_t refl[3] = {1, 1, -1};
    uint32_t n = 0;
    char buf[128];
    int fixed = 0;
    if (pwa_likelihood_create(&L) != PWA_SUCCESS) return 1;
    if (pwa_likelihood_init(L, 3, names, refl, 0, 2, 1.5) != PWA_SUCCESS) return 2;
    if (pwa_likelihood_nmb_pars(L, &n) != PWA_SUCCESS) return 3;
    printf("pars %u\n", n);
    if (pwa_likelihood_parameter(L, 0, buf, sizeof(buf), &fixed, 0, 0, 0) != PWA_SUCCESS) return 4;
    printf("first %s\n", buf);
    /* evaluation before finishInit is refused with a status and a message */
    double par[16] = {0}, f = 0, g[16];
    int st = pwa_likelihood_fdf(L, par, &f, g);
    printf("fdf status %d: %s\n", st, pwa_last_error());
    pwa_likelihood_destroy(L);
    if (st != PWA_ERROR_INVALID_STATE) return 5;
    /* decay amplitudes: a wave given as a plain C struct (spins doubled) */
    pwa_isobar* A = 0;
    pwa_isobar_wave w = {2, 1, 0, 1, 0, 2, 2, 2, 0, PWA_MASSDEP_RELATIVISTIC_BW, 0.769, 0.150, 1, 2, 0, 0};
    const double m[3] = {0.13957, 0.13957, 0.13957};
    const int32_t sp[3] = {0, 1, 0};
    double cg = 0;
    uint32_t terms = 0;
    if (pwa_isobar_create(&A) != PWA_SUCCESS) return 6;
    if (pwa_isobar_set_final_state(A, 3, m, sp, 0.13957) != PWA_SUCCESS) return 7;
    if (pwa_isobar_add_wave(A, &w) != PWA_SUCCESS) return 8;
    if (pwa_isobar_nmb_sym_terms(A, 0, &terms) != PWA_SUCCESS || terms != 2) return 9;
    w.M = 4; /* |M| > J */
    if (pwa_isobar_add_wave(A, &w) != PWA_ERROR_INVALID_ARGUMENT) return 10;
    printf("wave refused: %s\n", pwa_last_error());
    if (pwa_clebsch_gordan(2, 2, 2, -2, 0, 0, &cg) != PWA_SUCCESS) return 11;
    printf("cg %.6f\n", cg);  /* (1 1 1 -1 | 0 0) = 1/sqrt(3) */
    pwa_isobar_destroy(A);
    return (cg > 0.577 && cg < 0.578) ? 0 : 12;
}
"""


def test_header_compiles_and_c_program_runs(tmp_path):
    gcc = shutil.which("gcc")
    if gcc is None:
        pytest.skip("no C compiler")
    lib = os.path.join(LIBDIR, "libpwa_gb300.so")
    if not os.path.exists(lib):
        pytest.skip("library not built")
    cuda_inc = "/usr/local/cuda/include"
    hdr = os.path.join(INC, "pwa_gb300.h")
    for std, comp in (("-std=c99", gcc), ("-std=c++17", shutil.which("g++") or gcc)):
        r = subprocess.run([comp, std, "-Wall", "-Werror", "-fsyntax-only", "-x", "c" if "c99" in std else "c++",
                            hdr], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
    src = tmp_path / "main.c"
    src.write_text(PROGRAM)
    exe = tmp_path / "main"
    r = subprocess.run([gcc, "-std=c99", "-I", INC, str(src), "-L", LIBDIR, "-lpwa_gb300",
                        "-Wl,-rpath," + LIBDIR, "-o", str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, (r.returncode, r.stdout, r.stderr)
    lines = r.stdout.splitlines()
    # rank 2: r0 over (2 pos: 1 real + 1 complex = 3) + (1 neg: 1 real) = 4;
    # r1: the neg wave (index 0 < rank 1) is absent, pos: wave 0 absent,
    # wave 1 real = 1; + flat = 1  ->  6
    assert lines[0] == "pars 6"
    assert lines[1].startswith("first V0_")
    assert lines[2].startswith("fdf status %d" % 2)
