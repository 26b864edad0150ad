"""Build the engine's shared library ``leniax_gb300/_lgx.so`` for sm_103a.

Each ``csrc/*.cu`` translation unit is compiled in parallel with nvcc, then
linked into one shared library exposing the C ABI of
``include/lenia_gb300.h``.  Run ``python -m leniax_gb300.build`` (or
``__graft_entry__.build()``).  Outputs are in-tree and git-ignored.
"""
import concurrent.futures
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, 'csrc')
OBJ = os.path.join(HERE, '_build')
LIB = os.path.join(HERE, '_lgx.so')

ARCH = ['-gencode', 'arch=compute_103a,code=sm_103a']
NVCC_FLAGS = ['-O3', '-lineinfo', '-std=c++17', '--expt-relaxed-constexpr', '-Xcompiler', '-fPIC',
              '-Xcompiler', '-fvisibility=hidden', '-Xptxas', '-warn-spills']


def nvcc_path():
    for cand in (os.environ.get('NVCC'), shutil.which('nvcc'), '/usr/local/cuda/bin/nvcc'):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError('nvcc not found: the engine needs the CUDA toolkit to build')


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith('.cu'))


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose=False, force=False, extra_flags=()):
    """Compile and link; returns the library path."""
    nvcc = nvcc_path()
    os.makedirs(OBJ, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(('.cuh', '.h'))]
    headers.append(os.path.join(os.path.dirname(HERE), 'include', 'lenia_gb300.h'))
    jobs = []
    objs = []
    for src in sources():
        obj = os.path.join(OBJ, os.path.basename(src)[:-3] + '.o')
        objs.append(obj)
        if force or _stale(obj, [src] + headers):
            cmd = [nvcc] + ARCH + NVCC_FLAGS + list(extra_flags) + ['-c', src, '-o', obj]
            jobs.append(cmd)

    def run(cmd):
        p = subprocess.run(cmd, capture_output=True, text=True)
        return cmd, p

    if jobs:
        with concurrent.futures.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            for cmd, p in ex.map(run, jobs):
                if verbose or p.returncode != 0:
                    sys.stderr.write(' '.join(cmd) + '\n' + p.stdout + p.stderr)
                if p.returncode != 0:
                    raise RuntimeError(f'nvcc failed for {cmd[-3]}')
    if force or jobs or _stale(LIB, objs):
        tmp = LIB + '.tmp'
        cmd = [nvcc] + ARCH + ['-shared', '-o', tmp] + objs
        p = subprocess.run(cmd, capture_output=True, text=True)
        if p.returncode != 0:
            sys.stderr.write(' '.join(cmd) + '\n' + p.stdout + p.stderr)
            raise RuntimeError('link failed')
        os.replace(tmp, LIB)
    return LIB


if __name__ == '__main__':
    build(verbose='-v' in sys.argv, force='-f' in sys.argv)
    print(LIB)
