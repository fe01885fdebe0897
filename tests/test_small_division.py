"""The pull-push kernels divide by sample counts and weight sums n <= 16, and by the constant 3.14
of pull.comp's radius, as RN(q + r R) with R = RN(1/d), q = RN(x R) and the exact residual
r = x - q d (one FMA): Markstein's correction. This test proves on the CPU that the sequence equals
IEEE single-precision x / d for every float significand and each of those divisors (x in [1, 2);
other binades scale exactly), so the kernels that use it stay bit-exact with the shaders' divisions."""
import subprocess

SRC = r"""
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>
int main(void) {
    long bad = 0;
    for (int n = 1; n <= 17; ++n) {
        const float fn = n == 17 ? 3.14f : (float)n;
        volatile float rr = 1.0f / fn;
        const float R = rr;
        for (uint32_t m = 0; m < (1u << 23); ++m) {
            const uint32_t bits = 0x3f800000u | m;
            float x;
            memcpy(&x, &bits, 4);
            volatile float q = x * R;
            const float r = fmaf(-q, fn, x);
            const float got = fmaf(r, R, q);
            volatile float want = x / fn;
            const float w = want;
            if (memcmp(&got, &w, 4) != 0) ++bad;
        }
    }
    printf("%ld\n", bad);
    return 0;
}
"""


def test_reciprocal_correction_equals_ieee_division(tmp_path):
    src = tmp_path / "div.c"
    src.write_text(SRC)
    exe = tmp_path / "div"
    subprocess.run(["gcc", "-O2", "-ffp-contract=off", str(src), "-o", str(exe), "-lm"], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.strip()
    assert out == "0", f"{out} mismatches"
