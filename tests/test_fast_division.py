"""The multiply-high divider of the mixed-radix transforms (csrc/fft_mixed.cuh,
make_fastdiv / FastDivU): the host-computed (m, s) give n / d exactly for
every divisor a tile can have (1..4096): every index below 2^16, the
multiples of d and their neighbours up to 2^31 (where a wrong rounding
shows first), and the largest indices below 2^31.

Host-only: a small host program compiled with nvcc prints (m, s) for every
divisor; the quotient (umulhi(n, m) + n) >> s is evaluated here in 64-bit
integers, as the device does in 32-bit (skipped when nvcc is absent)."""
import os
import shutil
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
FFT_MIXED_H = os.path.join(os.path.dirname(HERE), 'leniax_gb300', 'csrc', 'fft_mixed.cuh')

PROGRAM = r'''
#include <cstdio>
#include "%s"
int main() {
  for (unsigned d = 1; d <= 4096; ++d) {
    const lgx::FastDivU f = lgx::make_fastdiv(d);
    printf("%%u %%u %%u\n", d, f.m, f.s);
  }
  return 0;
}
'''


@pytest.mark.skipif(shutil.which('nvcc') is None, reason='needs nvcc')
def test_fast_division_is_exact(tmp_path):
    src = tmp_path / 'fd.cu'
    src.write_text(PROGRAM % FFT_MIXED_H)
    exe = tmp_path / 'fd'
    subprocess.run(['nvcc', '-std=c++17', '-gencode', 'arch=compute_103a,code=sm_103a', '-o', str(exe), str(src)],
                   check=True, capture_output=True)
    rows = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split()
    table = np.array(rows, dtype=np.uint64).reshape(-1, 3)
    assert len(table) == 4096
    small = np.arange(0, 1 << 16, dtype=np.uint64)
    big = np.array([2**31 - 1, 2**31 - 2, 2**30 + 12345, 1999999999], dtype=np.uint64)
    top = np.uint64(2**31 - 1)
    for d, m, s in table:
        assert m < (1 << 32)
        k = np.unique(np.linspace(1, int(top // d), 4096).astype(np.uint64))
        edges = np.concatenate([k * d - np.uint64(1), k * d, k * d + np.uint64(1)])
        x = np.concatenate([small, big, edges[edges <= top]])
        hi = (x * m) >> np.uint64(32)  # umulhi(n, m): n < 2^31, m < 2^32
        q = (hi + x) >> s
        assert np.array_equal(q, x // d), int(d)
