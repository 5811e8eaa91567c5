"""Builds libswm_gb300.so in-tree with nvcc for sm_103a (no CMake, no torch).

Each translation unit compiles in parallel; FP64 units that must round like
the FP64 restatement are compiled with -fmad=false.
"""
import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, 'csrc')
BUILD = os.path.join(HERE, '_build')
LIB = os.path.join(HERE, 'libswm_gb300.so')
ARCH = ['-gencode', 'arch=compute_103a,code=sm_103a']
UNITS = {
    'api.cu': [], 'setup.cu': [], 'plain.cu': ['-fmad=false'], 'tracer.cu': ['-fmad=false'],
    'sor.cu': ['-fmad=false'], 'fused.cu': [], 'march.cu': [], 'ensemble.cu': [], 'trc32.cu': [], 'helm.cu': ['-fmad=false'], 'diag.cu': ['-fmad=false'],
}


def nvcc():
    cand = os.path.join(os.environ.get('CUDA_HOME', '/usr/local/cuda'), 'bin', 'nvcc')
    return cand if os.path.exists(cand) else 'nvcc'


def _compile(src, extra):
    obj = os.path.join(BUILD, src.replace('.cu', '.o'))
    # SWM_GB300_NVCC_FLAGS: extra nvcc flags (e.g. -D tuning macros)
    extra = list(extra) + os.environ.get('SWM_GB300_NVCC_FLAGS', '').split()
    cmd = [nvcc(), *ARCH, '-O3', '-lineinfo', '-std=c++17', '-Xcompiler', '-fPIC,-ffp-contract=off', '-Xptxas', '-v',
           '--expt-relaxed-constexpr', *extra, '-c', os.path.join(CSRC, src), '-o', obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError('nvcc failed for %s:\n%s' % (src, r.stderr))
    return obj, r.stderr


def build(verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 2)) as ex:
        futs = {ex.submit(_compile, s, e): s for s, e in UNITS.items()}
        objs = []
        for f in cf.as_completed(futs):
            obj, log = f.result()
            objs.append(obj)
            if verbose:
                print(log)
    cmd = [nvcc(), *ARCH, '-shared', '-o', LIB, *sorted(objs)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError('link failed:\n' + r.stderr)
    return LIB


if __name__ == '__main__':
    print(build(verbose='-v' in sys.argv))
