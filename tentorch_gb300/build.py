'''
Build `libtentorch_gb300.so` in this directory: the host engine (C++) and the sm_103a kernels
(CUDA), compiled in parallel, one translation unit per process, and linked with nvcc.

    python tentorch_gb300/build.py          # or tentorch_gb300.build.build()

A unit is recompiled when it is older than its source or any header; the library is relinked when
any object changed.  Only `nvcc` and `g++` are needed (no cmake, no torch extension machinery).
'''
import concurrent.futures
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, 'csrc')
OBJ = os.path.join(HERE, '_build')
LIBRARY = os.path.join(HERE, 'libtentorch_gb300.so')
INCLUDE = os.path.join(os.path.dirname(HERE), 'include')
ARCH = ['-gencode', 'arch=compute_103a,code=sm_103a']


def _cuda_home() -> str:
    nvcc = shutil.which('nvcc')
    if nvcc:
        return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))
    return os.environ.get('CUDA_HOME', '/usr/local/cuda')


def _nvcc() -> str:
    return shutil.which('nvcc') or os.path.join(_cuda_home(), 'bin', 'nvcc')


def _headers() -> list[str]:
    return glob.glob(os.path.join(CSRC, '*.h')) + glob.glob(os.path.join(INCLUDE, '*.h'))


def _command(source: str, obj: str) -> list[str]:
    if source.endswith('.cu'):
        return [_nvcc(), *ARCH, '-lineinfo', '-O3', '-std=c++17', '-Xcompiler', '-fPIC', '-Xptxas', '-v',
                f'-I{INCLUDE}', '-c', source, '-o', obj]
    return ['g++', '-O2', '-std=c++17', '-fPIC', '-Wall', '-Wno-sign-compare', f'-I{INCLUDE}',
            f'-I{os.path.join(_cuda_home(), "include")}', '-c', source, '-o', obj]


def _stale(source: str, obj: str, newest_header: float) -> bool:
    return not os.path.exists(obj) or os.path.getmtime(obj) < max(os.path.getmtime(source), newest_header)


def build(verbose: bool = False) -> str:
    '''Compile what is stale, link, and return the library path.'''
    os.makedirs(OBJ, exist_ok = True)
    sources = sorted(glob.glob(os.path.join(CSRC, '*.cu')) + glob.glob(os.path.join(CSRC, '*.cpp')))
    newest = max(os.path.getmtime(h) for h in _headers())
    jobs = []
    for src in sources:
        obj = os.path.join(OBJ, os.path.basename(src) + '.o')
        if _stale(src, obj, newest):
            jobs.append((src, obj))
    logs = {}
    with concurrent.futures.ThreadPoolExecutor(max_workers = max(1, min(len(jobs), os.cpu_count() or 4))) as pool:
        futures = {pool.submit(subprocess.run, _command(s, o), capture_output = True, text = True): (s, o)
                   for s, o in jobs}
        for future in concurrent.futures.as_completed(futures):
            src, _ = futures[future]
            result = future.result()
            logs[src] = result.stdout + result.stderr
            if result.returncode != 0:
                raise RuntimeError(f'compiling {os.path.basename(src)} failed:\n{logs[src]}')
    with open(os.path.join(OBJ, 'ptxas.log'), 'a') as handle:
        for src, text in logs.items():
            handle.write(f'== {os.path.basename(src)}\n{text}\n')
    objects = [os.path.join(OBJ, os.path.basename(s) + '.o') for s in sources]
    if jobs or not os.path.exists(LIBRARY) or os.path.getmtime(LIBRARY) < max(os.path.getmtime(o) for o in objects):
        link = [_nvcc(), *ARCH, '-shared', '-o', LIBRARY, *objects, '-lcublas', '-lcudart']
        result = subprocess.run(link, capture_output = True, text = True)
        if result.returncode != 0:
            raise RuntimeError(f'linking failed:\n{result.stdout}{result.stderr}')
    if verbose:
        for src, text in logs.items():
            print(f'== {os.path.basename(src)}\n{text}')
    return LIBRARY


if __name__ == '__main__':
    print(build(verbose = '--verbose' in sys.argv))
