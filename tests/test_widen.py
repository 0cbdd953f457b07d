"""The integer FP32 -> FP64 widening the CG vector kernels use (voxelfem_gb300/csrc/vfem_widen.h)
compiled for the host from the same header and checked against the C conversion for every one
of the 2^32 float bit patterns (NaNs: both results NaN with the same sign)."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PROGRAM = r"""
#include <stdio.h>
#include <string.h>
#include "vfem_widen.h"

int main(void) {
    unsigned long long bad = 0;
    for (unsigned long long i = 0; i <= 0xffffffffull; ++i) {
        const uint32_t b = (uint32_t)i;
        float f;
        memcpy(&f, &b, 4);
        const double r = (double)f;
        uint64_t want;
        memcpy(&want, &r, 8);
        const uint64_t got = vfem_widen_bits(b);
        const int nan_f = ((b >> 23) & 0xffu) == 0xffu && (b & 0x7fffffu);
        const int ok = nan_f ? ((got >> 52) & 0x7ffu) == 0x7ffu && (got & 0xfffffffffffffull) && (got >> 63) == (want >> 63)
                             : got == want;
        if (!ok) {
            if (bad < 4) printf("mismatch %08x: %016llx vs %016llx\n", b, (unsigned long long)got, (unsigned long long)want);
            ++bad;
        }
    }
    printf("mismatches %llu\n", bad);
    return bad != 0;
}
"""


@pytest.mark.skipif(shutil.which("gcc") is None, reason="needs gcc")
def test_widen_matches_c_conversion_for_every_float(tmp_path):
    src = tmp_path / "widen_check.c"
    exe = tmp_path / "widen_check"
    src.write_text(PROGRAM)
    subprocess.run(["gcc", "-O2", "-std=c99", "-I", os.path.join(ROOT, "voxelfem_gb300", "csrc"), str(src), "-o",
                    str(exe)], check=True)
    res = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert res.returncode == 0, res.stdout
    assert "mismatches 0" in res.stdout
