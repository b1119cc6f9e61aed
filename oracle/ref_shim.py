"""Import shim that makes the reference yaff importable in this container.

TEST INFRASTRUCTURE ONLY.  Used by tests/golden/make_golden.py and by CPU
tests that cross-check the oracle port against the real reference.  Nothing in
the product imports this module.

The reference needs ``molmod`` (units, logging) and ``h5py``, neither of which
is installed.  This shim registers small stand-ins for both, registers the
``yaff`` / ``yaff.pes`` / ``yaff.sampling`` packages as bare namespace packages
over the read-only checkout (so their heavy ``__init__`` files are not run),
and points ``yaff.pes.ext`` at the extension built by oracle/build_ref.sh.
The unit stand-ins are the harness constants of yaff_gb300.units.
"""
import contextlib
import os
import sys
import types

HERE = os.path.dirname(os.path.abspath(__file__))
REF_EXT_DIR = os.path.join(HERE, '_ref', 'pes')


def _reference_root():
    """The reference checkout: $YAFF_REFERENCE, else the one build_ref.sh
    compiled the extension from (recorded in _ref/REFERENCE_ROOT)."""
    root = os.environ.get('YAFF_REFERENCE')
    if root:
        return root
    rec = os.path.join(HERE, '_ref', 'REFERENCE_ROOT')
    if os.path.isfile(rec):
        with open(rec) as fh:
            return fh.read().strip()
    return ''


REF_ROOT = _reference_root()


def reference_available():
    """True when both the reference sources and its built extension exist."""
    if not os.path.isfile(os.path.join(REF_ROOT, 'yaff', 'pes', 'ff.py')):
        return False
    if not os.path.isdir(REF_EXT_DIR):
        return False
    return any(f.startswith('ext.') and f.endswith('.so') for f in os.listdir(REF_EXT_DIR))


class _Log(object):
    do_warning = False
    do_medium = False
    do_high = False
    do_debug = False
    do_low = False

    def __call__(self, *args, **kwargs):
        pass

    @contextlib.contextmanager
    def section(self, *args, **kwargs):
        yield

    def warn(self, *args, **kwargs):
        pass

    def hline(self, *args, **kwargs):
        pass

    def blank(self, *args, **kwargs):
        pass


class _Timer(object):
    @contextlib.contextmanager
    def section(self, *args, **kwargs):
        yield


def _pkg(name, path):
    mod = types.ModuleType(name)
    mod.__path__ = [path] if isinstance(path, str) else list(path)
    sys.modules[name] = mod
    parent, _, child = name.rpartition('.')
    if parent:
        setattr(sys.modules[parent], child, mod)
    return mod


def import_reference():
    """Register the stand-ins and return the reference ``yaff`` package.

    After this call ``import yaff.pes.ff``, ``yaff.pes.nlist``,
    ``yaff.system`` and ``yaff.sampling.verlet`` import the reference code.
    """
    if 'yaff.pes.ext' in sys.modules:
        return sys.modules['yaff']
    if not reference_available():
        raise ImportError('reference yaff (sources + oracle/_ref build) not available')
    repo = os.path.dirname(HERE)
    if repo not in sys.path:
        sys.path.insert(0, repo)
    from yaff_gb300 import units

    molmod = _pkg('molmod', [])
    mu = types.ModuleType('molmod.units')
    for k in units.__all__:
        setattr(mu, k, getattr(units, k))
    mu.__all__ = list(units.__all__)
    mu.parse_unit = lambda s: eval(s, {}, {k: getattr(units, k) for k in units.__all__})
    sys.modules['molmod.units'] = mu
    mc = types.ModuleType('molmod.constants')
    mc.boltzmann = units.boltzmann
    mc.__all__ = ['boltzmann']
    sys.modules['molmod.constants'] = mc
    ml = types.ModuleType('molmod.log')
    ml.ScreenLog = object
    ml.TimerGroup = object
    sys.modules['molmod.log'] = ml
    molmod.units = mu
    molmod.constants = mc
    molmod.log = ml
    for k in units.__all__:
        setattr(molmod, k, getattr(units, k))
    sys.modules.setdefault('h5py', types.ModuleType('h5py'))

    yaff = _pkg('yaff', os.path.join(REF_ROOT, 'yaff'))
    yaff.__version__ = 'reference'
    ylog = types.ModuleType('yaff.log')
    ylog.log = _Log()
    ylog.timer = _Timer()
    ylog.__all__ = ['log', 'timer']
    sys.modules['yaff.log'] = ylog
    yaff.log = ylog
    _pkg('yaff.pes', [REF_EXT_DIR, os.path.join(REF_ROOT, 'yaff', 'pes')])
    _pkg('yaff.sampling', os.path.join(REF_ROOT, 'yaff', 'sampling'))
    import warnings
    warnings.filterwarnings('ignore', category=SyntaxWarning)
    import yaff.pes.ext  # noqa: F401  (the built extension)
    return yaff
