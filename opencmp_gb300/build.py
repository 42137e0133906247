"""Builds libopencmp_gpu.so in-tree for sm_103a (nvcc for the kernels, g++ for the host set-up).

The translation units compile in parallel; the shared library lands next to this file
(``opencmp_gb300/libopencmp_gpu.so``) so every process loads the in-tree build.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, 'csrc')
BUILD = os.path.join(HERE, '_build')
LIB = os.path.join(HERE, 'libopencmp_gpu.so')
NVCC = os.environ.get('NVCC', '/usr/local/cuda/bin/nvcc' if os.path.exists('/usr/local/cuda/bin/nvcc') else 'nvcc')
CUDA_INC = os.path.join(os.path.dirname(os.path.dirname(os.path.realpath(NVCC))), 'include') \
    if os.path.isabs(NVCC) else '/usr/local/cuda/include'
ARCH = ['-gencode', 'arch=compute_103a,code=sm_103a']
CU_FLAGS = ARCH + ['-O3', '-lineinfo', '-std=c++17', '-Xcompiler', '-fPIC', '--expt-relaxed-constexpr',
                   '-I' + os.path.join(os.path.dirname(os.path.abspath(__file__)), '_build')]
CXX_FLAGS = ['-O2', '-std=c++17', '-fPIC', '-I' + CUDA_INC]


def sources():
    cu = sorted(f for f in os.listdir(CSRC) if f.endswith('.cu'))
    cpp = sorted(f for f in os.listdir(CSRC) if f.endswith('.cpp'))
    return cu, cpp


def _newer(out, deps):
    return os.path.exists(out) and all(os.path.getmtime(out) >= os.path.getmtime(d) for d in deps)


GEN_HEADER = os.path.join(BUILD, 'ocmp_terms_gen.h')


def _generate_terms(verbose: bool):
    """Compile and run the term-table generator (ocmp_host.cpp, OCMP_TERM_GENERATOR), which writes
    the straight-line element-matrix code the double-float kernel includes."""
    src = os.path.join(CSRC, 'ocmp_host.cpp')
    deps = [src, os.path.join(CSRC, 'ocmp_internal.h')]
    if _newer(GEN_HEADER, deps):
        return
    exe = os.path.join(BUILD, 'ocmp_termgen')
    # only the table builders run; the kernel launchers the TU references are never called
    cmd = [NVCC, '-std=c++17', '-O1', '-DOCMP_TERM_GENERATOR', '-x', 'c++', src, '-o', exe,
           '-Xlinker', '--unresolved-symbols=ignore-all']
    if verbose:
        print(' '.join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError('term generator build failed:\n{}{}'.format(r.stdout, r.stderr))
    r = subprocess.run([exe, GEN_HEADER + '.tmp'], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError('term generator failed ({}): {}'.format(r.returncode, r.stderr))
    os.replace(GEN_HEADER + '.tmp', GEN_HEADER)


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    if force and os.path.exists(GEN_HEADER):
        os.remove(GEN_HEADER)
    _generate_terms(verbose)
    cu, cpp = sources()
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(('.h', '.cuh'))]
    headers.append(os.path.join(HERE, '..', 'include', 'opencmp_gpu.h'))
    headers.append(GEN_HEADER)
    jobs, objs = [], []
    for f in cu + cpp:
        src = os.path.join(CSRC, f)
        obj = os.path.join(BUILD, f + '.o')
        objs.append(obj)
        if not force and _newer(obj, [src] + headers):
            continue
        if f.endswith('.cu'):
            cmd = [NVCC] + CU_FLAGS + ['-c', src, '-o', obj]
        else:
            cmd = ['g++'] + CXX_FLAGS + ['-c', src, '-o', obj]
        jobs.append(cmd)

    def run(cmd):
        if verbose:
            print(' '.join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError('build failed: {}\n{}{}'.format(' '.join(cmd), r.stdout, r.stderr))
        return r.stderr

    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for _ in ex.map(run, jobs):
            pass
    if jobs or force or not _newer(LIB, objs):
        run([NVCC] + ARCH + ['-shared', '-o', LIB] + objs + ['-lcudart'])
    return LIB


if __name__ == '__main__':
    print(build(force='--force' in sys.argv, verbose=True))
