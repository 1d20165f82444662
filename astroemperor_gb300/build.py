"""Build the CUDA shared library ``libemp_gpu.so`` in-tree (sm_103a only).

Each ``csrc/*.cu`` translation unit is compiled by its own ``nvcc`` process
(in parallel) and the objects are linked into
``astroemperor_gb300/_lib/libemp_gpu.so``.  A build is skipped when the
library was built from the same sources: a SHA-256 over every source and
header, the compiler flags and the machine type, written next to the
library, must match (file times are not trusted: a copied tree keeps a
library built elsewhere).  ``build`` prints whether it compiled.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import hashlib
import os
import platform
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, 'csrc')
INCLUDE = os.path.join(ROOT, 'include')
OUTDIR = os.path.join(PKG, '_lib')
LIB = os.path.join(OUTDIR, 'libemp_gpu.so')
ARCH = ['-gencode', 'arch=compute_103a,code=sm_103a']


def nvcc_path() -> str:
    for cand in (os.environ.get('NVCC'), shutil.which('nvcc'), '/usr/local/cuda/bin/nvcc'):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError('nvcc not found: the CUDA toolkit is required to build libemp_gpu.so')


def _sources():
    return sorted(glob.glob(os.path.join(CSRC, '*.cu')))


def _deps():
    return _sources() + glob.glob(os.path.join(CSRC, '*.cuh')) + glob.glob(os.path.join(INCLUDE, '*.h'))


STAMP = LIB + '.sha256'
BASE_FLAGS = ['-O3', '-lineinfo', '-std=c++17', '-Xcompiler', '-fPIC']


def source_hash(extra_flags=None) -> str:
    """SHA-256 of the sources, headers, flags and machine type."""
    h = hashlib.sha256()
    for p in sorted(_deps()):
        h.update(os.path.relpath(p, ROOT).encode())
        with open(p, 'rb') as f:
            h.update(f.read())
    h.update(' '.join(ARCH + BASE_FLAGS + list(extra_flags or [])).encode())
    h.update(platform.machine().encode())
    return h.hexdigest()


def up_to_date(extra_flags=None) -> bool:
    if not (os.path.exists(LIB) and os.path.exists(STAMP)):
        return False
    with open(STAMP) as f:
        return f.read().strip() == source_hash(extra_flags)


def build(force: bool = False, verbose: bool = False, extra_flags=None, quiet: bool = False) -> str:
    """Compile and link unless the library matches the sources; returns its path."""
    digest = source_hash(extra_flags)
    if not force and up_to_date(extra_flags):
        if not quiet:
            print(f'libemp_gpu.so up to date (sources {digest[:12]})')
        return LIB
    nvcc = nvcc_path()
    os.makedirs(OUTDIR, exist_ok=True)
    flags = ARCH + BASE_FLAGS + ['-I', INCLUDE, '-I', CSRC] + list(extra_flags or [])
    objs = []
    cmds = []
    for src in _sources():
        obj = os.path.join(OUTDIR, os.path.basename(src)[:-3] + '.o')
        objs.append(obj)
        cmds.append([nvcc, *flags, '-c', src, '-o', obj])

    def run(cmd):
        p = subprocess.run(cmd, capture_output=True, text=True)
        return cmd, p

    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(cmds), os.cpu_count() or 1))) as ex:
        for cmd, p in ex.map(run, cmds):
            if verbose or p.returncode != 0:
                sys.stderr.write(' '.join(cmd) + '\n' + p.stdout + p.stderr)
            if p.returncode != 0:
                raise RuntimeError(f'nvcc failed for {cmd[-3]}')
    link = [nvcc, *ARCH, '-shared', '-cudart', 'static', '-o', LIB + '.tmp', *objs]
    p = subprocess.run(link, capture_output=True, text=True)
    if p.returncode != 0:
        sys.stderr.write(' '.join(link) + '\n' + p.stdout + p.stderr)
        raise RuntimeError('link of libemp_gpu.so failed')
    os.replace(LIB + '.tmp', LIB)
    with open(STAMP, 'w') as f:
        f.write(digest + '\n')
    for o in objs:
        try:
            os.remove(o)
        except OSError:
            pass
    if not quiet:
        print(f'libemp_gpu.so compiled (sources {digest[:12]}, {platform.machine()})')
    return LIB


if __name__ == '__main__':
    print(build(force='--force' in sys.argv, verbose='-v' in sys.argv))
