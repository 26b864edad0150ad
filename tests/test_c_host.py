"""A C host (no Python, no torch) compiles against include/lenia_gb300.h as
C99, links the engine library and creates, queries and destroys plans
through the C ABI; model validation answers with the header's status codes
(no device work: runs without a GPU)."""
import ctypes
import os
import re
import shutil
import subprocess

import pytest

from leniax_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

HOST_C = r'''
#include <stdio.h>
#include <string.h>
#include "lenia_gb300.h"

static int make(int nb_dims, int a, int b, int c, int nb_channels, lgx_plan** out) {
  /* leniax's aquarium topology, scaled down: 2 channels, 3 kernels, max_k 2 */
  static const int cin[3] = {0, 1, 1}, slot[3] = {0, 0, 1};
  static const int gf[3] = {LGX_GF_GAUSSIAN, LGX_GF_POLY_QUAD4, LGX_GF_STEP};
  lgx_model_desc d;
  memset(&d, 0, sizeof d);
  d.nb_dims = nb_dims;
  d.world[0] = a;
  d.world[1] = b;
  d.world[2] = c;
  d.nb_channels = nb_channels;
  d.nb_kernels = 3;
  d.max_k = 2;
  d.kernel_cin = cin;
  d.kernel_slot = slot;
  d.growth_fn = gf;
  d.state_fn = LGX_STATE_V1;
  d.weighted_average = 0;
  return lgx_plan_create(&d, out);
}

int main(void) {
  lgx_plan* p = NULL;
  int rc;
  if (lgx_version() != LGX_ABI_VERSION) return 10;
  rc = make(2, 128, 128, 0, 2, &p);
  if (rc != LGX_OK || !p) return 11;
  printf("2d engine=%d run_ws=%zu update_ws=%zu\n", lgx_select_engine(p, 2, 3, LGX_ENGINE_AUTO),
         lgx_run_workspace_bytes(p, 2, 3, 16, LGX_ENGINE_AUTO), lgx_update_workspace_bytes(p, 4));
  lgx_plan_destroy(p);
  p = NULL;
  rc = make(3, 48, 48, 48, 2, &p);
  if (rc != LGX_OK || !p) return 12;
  printf("3d engine=%d\n", lgx_select_engine(p, 1, 1, LGX_ENGINE_AUTO));
  lgx_plan_destroy(p);
  p = NULL;
  rc = make(2, 8192, 64, 0, 2, &p); /* sides up to 4096 */
  printf("big rc=%d plan=%d msg=%s\n", rc, p != NULL, lgx_last_error());
  rc = make(2, 64, 64, 0, 1, &p); /* kernel 1 reads channel 1 of 1 */
  printf("bad rc=%d plan=%d msg=%s\n", rc, p != NULL, lgx_last_error());
  return 0;
}
'''


def test_c_host_compiles_links_and_validates_plans(tmp_path):
    gcc = shutil.which('gcc')
    if gcc is None:
        pytest.skip('gcc not available')
    _lib.load()  # the library is built
    src = tmp_path / 'host.c'
    src.write_text(HOST_C)
    exe = tmp_path / 'host'
    so_dir = os.path.dirname(_lib.LIB_PATH)
    subprocess.run([gcc, '-std=c99', '-Wall', '-Wextra', '-Werror', '-I', os.path.join(ROOT, 'include'), str(src),
                    '-o', str(exe), _lib.LIB_PATH, f'-Wl,-rpath,{so_dir}'], check=True, capture_output=True, text=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True, timeout=120).stdout.splitlines()
    lines = dict(line.split(' ', 1) for line in out)
    fields = dict(kv.split('=', 1) for kv in lines['2d'].split())
    assert int(fields['engine']) == _lib.ENGINES['streamed']  # several channels at 128^2
    assert int(fields['run_ws']) > 0 and int(fields['update_ws']) > 0
    assert int(lines['3d'].split('=')[1]) == _lib.ENGINES['nd']
    assert lines['big'].startswith(f'rc={_lib.LGX_ERR_UNSUPPORTED} plan=0 msg=world axis 0')
    assert lines['bad'].startswith(f'rc={_lib.LGX_ERR_INVALID} plan=0 msg=kernel 1 reads channel 1 of 1')


def _mirrors():
    from leniax_gb300 import batch, grad, initializations, kernels
    return {'lgx_model_desc': _lib.ModelDesc, 'lgx_rollout': _lib.Rollout, 'lgx_adjoint_job': grad.AdjointJob,
            'lgx_ring_batch': kernels.RingBatchC.get(), 'lgx_init_job': initializations.InitJobC,
            'lgx_batch_class': batch.BatchClassC, 'lgx_batch_job': batch.BatchJobC}


def test_ctypes_mirrors_match_the_header_layout(tmp_path):
    # every struct of include/lenia_gb300.h against its ctypes mirror: the
    # same field names, offsets and size (the engine reads them through a bare pointer)
    gcc = shutil.which('gcc')
    if gcc is None:
        pytest.skip('gcc not available')
    mirrors = _mirrors()
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "lenia_gb300.h"', 'int main(void) {']
    for cname, cls in mirrors.items():
        lines.append(f'  printf("{cname} sizeof %zu\\n", sizeof({cname}));')
        for fname, _ in cls._fields_:
            lines.append(f'  printf("{cname} {fname} %zu\\n", offsetof({cname}, {fname}));')
    lines += ['  return 0;', '}']
    src = tmp_path / 'layout.c'
    src.write_text('\n'.join(lines) + '\n')
    exe = tmp_path / 'layout'
    subprocess.run([gcc, '-std=c99', '-Wall', '-Werror', '-I', os.path.join(ROOT, 'include'), str(src), '-o',
                    str(exe)], check=True, capture_output=True, text=True)
    got = {}
    for line in subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.splitlines():
        cname, fname, val = line.split()
        got[(cname, fname)] = int(val)
    header = open(os.path.join(ROOT, 'include', 'lenia_gb300.h')).read()
    for cname, cls in mirrors.items():
        assert got[(cname, 'sizeof')] == ctypes.sizeof(cls), cname
        for fname, _ in cls._fields_:
            assert got[(cname, fname)] == getattr(cls, fname).offset, (cname, fname)
        # and the mirror lists every field the header declares
        body = header[header.index(f'typedef struct {cname} {{'):]
        body = body[:body.index(f'}} {cname};')]
        declared = set()
        for stmt in re.sub(r'/\*.*?\*/', '', body[body.index('{') + 1:], flags=re.S).split(';'):
            for part in filter(None, (p.strip() for p in stmt.split(','))):
                declared.add(re.search(r'(\w+)\s*(?:\[\d+\])?$', part).group(1))
        assert declared == {f for f, _ in cls._fields_}, (cname, declared ^ {f for f, _ in cls._fields_})
