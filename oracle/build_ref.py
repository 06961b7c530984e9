"""Build recipe for ``oracle/_ref`` -- ORACLE / test infrastructure only.

Compiles the reference's own CPU operator so tests can pin the restatement in
``oracle/commit_oracle.c`` against it and the benchmark can time it as the reference
CPU baseline.  Outputs go to ``oracle/_ref/`` only (git-ignored).

1. The reference writes its C operator from a Python template (setup_operator.py:938-947,
   ``write_operator_c_file()``, which writes ``commit/operator/operator_c.c`` relative to
   the working directory).  We run that generator with the working directory set to
   ``oracle/_ref/gen`` so the generated file lands there.  Needs the reference tree
   (``COMMIT_REFERENCE`` or /root/reference); skipped when absent if a generated file
   is already present (the file then travels with the repository copy).
2. gcc compiles it with the reference's flags (setup.py:38-43: ``-w -O3 -Ofast``) into
   ``oracle/_ref/libcommit_ref_operator.so``; rebuilt when the library is missing or was
   built for another machine architecture.
3. ``oracle/_ref/libt2d_ref.so``: the reference's streamline voxeliser
   (commit/trk2dictionary/trk2dictionary_c.cpp, compiled from the reference tree with its
   Vector.h / ProgressBar.h and the numpy / Python headers it includes, no libpython
   needed) plus ``oracle/t2d_ref_driver.cpp``, a C entry point that runs it on a .trk
   file.  ``-ffp-contract=off`` keeps the FP64 geometry free of fused multiply-adds on
   every architecture.  Needs the reference tree; skipped without it.
4. With ``--python`` (needs Cython and the reference tree): Cython-compiles
   commit/proximals.pyx into ``oracle/_ref/py/commit/`` and writes a two-function
   ``dicelib.ui`` logger stub, so the reference ``commit/solvers.py`` can be imported
   for golden-vector generation (``tests/golden/make_golden.py``).
"""
from __future__ import annotations

import os
import platform
import subprocess
import sys
import sysconfig

HERE = os.path.dirname(os.path.abspath(__file__))
REF_OUT = os.path.join(HERE, '_ref')
GEN = os.path.join(REF_OUT, 'gen')
GEN_C = os.path.join(GEN, 'commit', 'operator', 'operator_c.c')
LIB = os.path.join(REF_OUT, 'libcommit_ref_operator.so')
ARCH_TAG = os.path.join(REF_OUT, 'lib_arch.txt')
PY_DIR = os.path.join(REF_OUT, 'py')


def reference_root() -> str | None:
    root = os.environ.get('COMMIT_REFERENCE', '/root/reference')
    return root if os.path.exists(os.path.join(root, 'setup_operator.py')) else None


def generate() -> bool:
    root = reference_root()
    if root is None:
        return os.path.exists(GEN_C)
    os.makedirs(os.path.dirname(GEN_C), exist_ok=True)
    code = ('import sys, os; sys.path.insert(0, %r); os.chdir(%r); '
            'import setup_operator; setup_operator.write_operator_c_file()') % (root, GEN)
    subprocess.run([sys.executable, '-c', code], check=True)
    return os.path.exists(GEN_C)


def compile_operator() -> bool:
    if not os.path.exists(GEN_C):
        return False
    arch = platform.machine()
    fresh = (os.path.exists(LIB) and os.path.exists(ARCH_TAG) and open(ARCH_TAG).read().strip() == arch
             and os.path.getmtime(LIB) >= os.path.getmtime(GEN_C))
    if fresh:
        return True
    cmd = ['gcc', '-w', '-O3', '-Ofast', '-shared', '-fPIC', '-o', LIB + '.tmp', GEN_C, '-lpthread']
    subprocess.run(cmd, check=True)
    os.replace(LIB + '.tmp', LIB)
    with open(ARCH_TAG, 'w') as f:
        f.write(arch)
    return True


DICELIB_STUB = '''"""Stand-in for dicelib.ui used only to import the reference modules for golden vectors."""
class _Logger:
    def __init__(self, name):
        self.name = name
    def error(self, msg, *a, **k):
        raise RuntimeError(msg)
    def _quiet(self, *a, **k):
        return None
    warning = info = subinfo = debug = _quiet


def setup_logger(name, *a, **k):
    return _Logger(name)
'''


def build_python() -> bool:
    root = reference_root()
    if root is None:
        return False
    try:
        import numpy
    except ImportError:
        return False
    os.makedirs(os.path.join(PY_DIR, 'commit'), exist_ok=True)
    os.makedirs(os.path.join(PY_DIR, 'dicelib'), exist_ok=True)
    with open(os.path.join(PY_DIR, 'dicelib', '__init__.py'), 'w') as f:
        f.write('')
    with open(os.path.join(PY_DIR, 'dicelib', 'ui.py'), 'w') as f:
        f.write(DICELIB_STUB)
    with open(os.path.join(PY_DIR, 'commit', '__init__.py'), 'w') as f:
        f.write('')
    c_out = os.path.join(GEN, 'proximals.c')
    subprocess.run([sys.executable, '-m', 'cython', '-3', '-o', c_out, os.path.join(root, 'commit', 'proximals.pyx')],
                   check=True)
    ext = sysconfig.get_config_var('EXT_SUFFIX')
    so = os.path.join(PY_DIR, 'commit', 'proximals' + ext)
    inc = sysconfig.get_paths()['include']
    subprocess.run(['gcc', '-w', '-O2', '-shared', '-fPIC', '-I', inc, '-I', numpy.get_include(), '-o', so, c_out],
                   check=True)
    return True


T2D_LIB = os.path.join(REF_OUT, 'libt2d_ref.so')


def compile_trk2dictionary() -> bool:
    root = reference_root()
    if root is None:
        return False
    try:
        import numpy
    except ImportError:
        return False
    src_dir = os.path.join(root, 'commit', 'trk2dictionary')
    src = os.path.join(src_dir, 'trk2dictionary_c.cpp')
    drv = os.path.join(HERE, 't2d_ref_driver.cpp')
    if not os.path.exists(src):
        return False
    os.makedirs(REF_OUT, exist_ok=True)
    inc = sysconfig.get_paths()['include']
    cmd = ['g++', '-O2', '-ffp-contract=off', '-w', '-shared', '-fPIC', '-I', numpy.get_include(), '-I', inc,
           '-I', src_dir, '-o', T2D_LIB + '.tmp', src, drv, '-lpthread']
    if subprocess.run(cmd).returncode != 0:
        return False
    os.replace(T2D_LIB + '.tmp', T2D_LIB)
    return True


def main(argv=None) -> int:
    argv = sys.argv[1:] if argv is None else argv
    ok = generate() and compile_operator()
    print('oracle/_ref operator:', 'built' if ok else 'unavailable (no reference tree and no generated source)')
    print('oracle/_ref trk2dictionary:', 'built' if compile_trk2dictionary() else 'unavailable (no reference tree)')
    if '--python' in argv:
        print('oracle/_ref python modules:', 'built' if build_python() else 'unavailable')
    return 0


if __name__ == '__main__':
    sys.exit(main())
