"""The C-ABI from a C99 program: the public header compiles as C, the program
links against libvegasgb.so and calls entry points that need no GPU (NVRTC
compile check, argument validation, error strings)."""

import os
import shutil
import subprocess

import pytest

from conftest import ROOT

C_CLIENT = r"""
#include <stdio.h>
#include "vegasflow_gb300.h"

int main(void) {
  char log[4096];
  const char* src =
      "__device__ vf_real f(const vf_real* x, int n, vf_real w, const double* p) { return x[0] * w; }";
  if (vf_version() < 1) return 1;
  if (vf_jit_check(src, "f", VF_ALG_VEGAS, VF_PREC_F32, 4, log, (int)sizeof(log)) != VF_OK) {
    printf("%s\n", log);
    return 2;
  }
  /* a NULL grid is rejected with VF_ERR_ARG and a message, nothing is launched */
  int rc = vf_sample(VF_ALG_VEGAS, VF_PREC_F64, NULL, 4, 10, 0, 0.1, NULL, NULL, 1.0, NULL, 1, 0,
                     VF_INT_SYMGAUSS, NULL, 1, 0, NULL, 1, NULL, NULL, NULL, NULL, NULL, NULL);
  if (rc != VF_ERR_ARG || vf_last_error_string()[0] == '\0') return 3;
  /* more than 16 dimensions is unsupported */
  rc = vf_sample(VF_ALG_VEGAS, VF_PREC_F64, NULL, 17, 10, 0, 0.1, NULL, NULL, 1.0, NULL, 1, 0,
                 VF_INT_SYMGAUSS, NULL, 1, 0, NULL, 1, NULL, NULL, NULL, NULL, NULL, NULL);
  if (rc != VF_ERR_UNSUPPORTED) return 4;
  printf("ok\n");
  return 0;
}
"""


def test_c_program_links_and_calls_the_abi(tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    from vegasflow_gb300.build import BUILD, LIB, build

    if not os.path.exists(LIB):
        build()
    src = tmp_path / "client.c"
    src.write_text(C_CLIENT)
    exe = tmp_path / "client"
    subprocess.run([cc, "-std=c99", "-Wall", "-Werror", f"-I{os.path.join(ROOT, 'include')}", str(src),
                    f"-L{BUILD}", "-lvegasgb", f"-Wl,-rpath,{BUILD}", "-o", str(exe)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and r.stdout.strip() == "ok", (r.returncode, r.stdout, r.stderr)
