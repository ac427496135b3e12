'''
Compile the reference engine (Jumqyc/TenTorch) from its own C++ sources, where they lie, into
``oracle/_ref/``.  Test infrastructure only: the compiled reference is the checker that the oracle
restatement and the golden fixtures are pinned against; nothing in the product loads it.

Two shared objects come out:

- ``oracle/_ref/ext/symmetry_ext.so``: the reference's own pybind11 module (``tentorch/_ext/
  bindings.cpp`` and the sources listed in ``tentorch/_ext/build.py:13-29``), so that
  ``oracle.ref_import.reference()`` can import the unmodified Python package on top of it.
- ``oracle/_ref/dump/ref_plan_dump.so``: ``oracle/ref_plan_dump.cpp`` linked against the same
  reference objects, which returns the per-step regrouping plans (``exchange_regrouping`` /
  ``bend_regrouping``, ``tentorch/tensors/regroup.h:69-96``) as plain Python data.  The plans are
  not bound by the reference's own module.

Recipe differences from the reference's ``tentorch/_ext/build.py:115-146``: ``-std=c++20`` is added
(torch's loader defaults to c++17 and ``fibonacci.cpp`` needs ``std::numbers``), and ``pch.h`` is
force-included as a plain header instead of a precompiled one.  The reference tree is read only; all
outputs go under ``oracle/_ref``.

Usage: ``python oracle/build_ref.py --reference <checkout>`` or with ``TENTORCH_REFERENCE`` set
(about two minutes on 8 cores).  It runs only where a reference checkout is named and present.
'''
import glob
import os
import sys

# the reference checkout: from --reference, or the TENTORCH_REFERENCE environment variable
REFERENCE = os.environ.get('TENTORCH_REFERENCE', '')
if '--reference' in sys.argv[:-1]:
    REFERENCE = sys.argv[sys.argv.index('--reference') + 1]
HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, '_ref')
EXT_DIR = os.path.join(OUT, 'ext')
DUMP_DIR = os.path.join(OUT, 'dump')

_UNITS = ('symmetry/cat/cat.cpp', 'symmetry/cat/group.cpp', 'symmetry/cat/abelian/abelian.cpp',
          'symmetry/cat/fibonacci/fibonacci.cpp', 'symmetry/cat/su2/su2.cpp',
          'symmetry/cat/su3/su3.cpp', 'symmetry/tree/tree.cpp', 'tensors/layout.cpp',
          'tensors/regroup.cpp', 'tensors/cache.cpp', 'tensors/place.cpp', 'tensors/tensor.cpp',
          'linalg/graded/contract.cpp', 'linalg/graded/svd.cpp', 'linalg/graded/compare.cpp',
          'linalg/graded/einsum.cpp')


def available() -> bool:
    '''Whether a reference checkout is named and its sources are present.'''
    return bool(REFERENCE) and os.path.isdir(os.path.join(REFERENCE, 'tentorch', 'tensors'))


def built() -> bool:
    '''Whether both shared objects exist.'''
    return (os.path.exists(os.path.join(EXT_DIR, 'symmetry_ext.so')) and
            os.path.exists(os.path.join(DUMP_DIR, 'ref_plan_dump.so')))


def _flags() -> list[str]:
    pch = os.path.join(REFERENCE, 'tentorch', '_ext', 'pch.h')
    return ['-O2', '-std=c++20', '-include', pch, '-w']


def build(verbose: bool = False):
    '''Compile both shared objects (ninja skips up-to-date units) and return the two modules.'''
    if not available():
        raise RuntimeError(f'the reference sources are not at {REFERENCE}')
    from torch.utils.cpp_extension import load
    os.makedirs(EXT_DIR, exist_ok = True)
    os.makedirs(DUMP_DIR, exist_ok = True)
    os.environ.setdefault('MAX_JOBS', str(os.cpu_count() or 4))
    root = os.path.join(REFERENCE, 'tentorch')
    sources = [os.path.join(root, '_ext', 'bindings.cpp')] + [os.path.join(root, u) for u in _UNITS]
    ext = load(name = 'symmetry_ext', sources = sources, extra_cflags = _flags(),
               build_directory = EXT_DIR, verbose = verbose)
    # the dump module reuses the engine objects compiled above, all but the reference's bindings
    objects = [os.path.join(EXT_DIR, os.path.splitext(os.path.basename(u))[0] + '.o') for u in _UNITS]
    dump = load(name = 'ref_plan_dump', sources = [os.path.join(HERE, 'ref_plan_dump.cpp')],
                extra_cflags = _flags() + [f'-I{root}'], extra_ldflags = objects,
                build_directory = DUMP_DIR, verbose = verbose)
    return ext, dump


if __name__ == '__main__':
    build(verbose = '--verbose' in sys.argv)
    print('built', sorted(glob.glob(os.path.join(OUT, '*', '*.so'))))
