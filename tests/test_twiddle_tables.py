"""The compile-time FFT twiddle tables (csrc/fft.cuh, kTwiddles<N, G>) equal
the float32 rounding of cos / sin of their angles, entry by entry.

The tables replace a per-block double-precision sincospi fill; this pins them
to the same values.  Host-only: the constexpr tables are evaluated by a small
host program compiled with nvcc (skipped when nvcc is absent)."""
import os
import shutil
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
FFT_H = os.path.join(os.path.dirname(HERE), 'leniax_gb300', 'csrc', 'fft.cuh')
SETS = [(32, 4), (64, 4), (128, 8), (256, 8), (256, 16), (512, 16), (64, 2), (32, 2)]

PROGRAM = r'''
#include <cstdio>
#include "%s"
using namespace lgx;
template <int N, int G> void dump() {
  static constexpr TwiddleTables<N, G> t{};
  for (int i = 0; i < 3 * N; ++i) printf("%%d %%d %%d %%a %%a\n", N, G, i, t.v[i].x, t.v[i].y);
}
int main() { %s return 0; }
'''


def _index_sets(N, G):
    P = N // G
    Q = P // G

    def pairs(t, q):
        if Q == 1:
            return t
        m = t + G * (q >> 1)
        return 2 * m + (q & 1)

    def mirror(t, q):
        if Q == 1:
            return t
        m = t + G * (q >> 1)
        if m == 0:
            return P // 2 if q & 1 else 0
        return P - m if q & 1 else m

    return pairs, mirror


@pytest.mark.skipif(shutil.which('nvcc') is None, reason='needs nvcc')
def test_compile_time_twiddles_match_float32_cos_sin(tmp_path):
    calls = ' '.join(f'dump<{n}, {g}>();' for n, g in SETS)
    src = tmp_path / 'tw.cu'
    src.write_text(PROGRAM % (FFT_H, calls))
    exe = tmp_path / 'tw'
    subprocess.run(['nvcc', '-std=c++17', '--expt-relaxed-constexpr', '-gencode', 'arch=compute_103a,code=sm_103a',
                    '-o', str(exe), str(src)], check=True, capture_output=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split('\n')
    n_entries = 0
    for line in out:
        if not line:
            continue
        N, G, i, x, y = line.split()
        N, G, i = int(N), int(G), int(i)
        pairs, mirror = _index_sets(N, G)
        tab, j = divmod(i, N)
        t, k2, kk, q = j % G, j // G, (j // G) % G, j // (G * G)
        m = [(t * k2) % N, (pairs(t, q) * kk) % N, (mirror(t, q) * kk) % N][tab]
        ang = 2 * np.pi * m / N
        # exact zeros at the quarter points (as sincospi gives them)
        ref_c = np.float32(0.0) if (4 * m) % N == 0 and (4 * m // N) % 2 == 1 else np.float32(np.cos(ang))
        ref_s = np.float32(0.0) if (2 * m) % N == 0 else np.float32(-np.sin(ang))
        assert np.float32(float.fromhex(x)) == ref_c, (N, G, i, x, ref_c)
        assert np.float32(float.fromhex(y)) == ref_s, (N, G, i, y, ref_s)
        n_entries += 1
    assert n_entries == sum(3 * n for n, _ in SETS)
