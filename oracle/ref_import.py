'''
Import the unmodified reference Python package (Jumqyc/TenTorch) on top of the engine that
``oracle/build_ref.py`` compiled from the reference's own sources.  Test infrastructure only: the
golden-fixture script uses it to produce reference outputs; the product never imports it.

The reference's ``tentorch/_ext/__init__.py:33-50`` would compile its engine into the (read-only)
reference tree, so this module registers ``tentorch._ext`` itself, re-exporting the compiled
module's names exactly as that file does (``tentorch/_ext/__init__.py:61-104``), and then imports the
rest of the package from the reference checkout unchanged.
'''
import importlib.util
import os
import sys
import types

from oracle import build_ref


def reference():
    '''The reference ``tentorch`` package and the plan-dump module, building them when missing.'''
    if 'tentorch' in sys.modules and hasattr(sys.modules['tentorch'], 'einsum'):
        return sys.modules['tentorch'], sys.modules['ref_plan_dump']
    import torch  # noqa: F401  (the engine hands at::Tensor objects to Python)
    if not build_ref.built():
        build_ref.build()

    def load(name, path):
        spec = importlib.util.spec_from_file_location(name, path)
        module = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(module)
        sys.modules[name] = module
        return module

    ext = load('symmetry_ext', os.path.join(build_ref.EXT_DIR, 'symmetry_ext.so'))
    dump = load('ref_plan_dump', os.path.join(build_ref.DUMP_DIR, 'ref_plan_dump.so'))
    shim = types.ModuleType('tentorch._ext')
    shim.__path__ = [os.path.join(build_ref.REFERENCE, 'tentorch', '_ext')]
    for name in dir(ext):
        if not name.startswith('__'):
            setattr(shim, name, getattr(ext, name))
    shim._engine = ext
    shim.Sector = tuple[int, ...]
    sys.modules['tentorch._ext'] = shim
    if build_ref.REFERENCE not in sys.path:
        sys.path.insert(0, build_ref.REFERENCE)
    import tentorch
    return tentorch, dump
