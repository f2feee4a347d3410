"""Import harness for the reference Spitfire (test infrastructure; runs only where the reference sources exist).

The reference package does not import as shipped here: ``spitfire/__init__.py:5-31`` pulls in Cantera and
``chemistry/reactors.py:24`` imports matplotlib, neither of which is installed. This harness

* registers empty ``spitfire``, ``spitfire.time``, ``spitfire.chemistry`` and ``spitfire.griffon`` packages,
* maps ``spitfire.griffon.griffon`` to the reference Griffon built unmodified by ``make -C oracle ref``
  (``oracle/_ref/griffon.*.so``),
* stubs ``matplotlib.pyplot`` and ``spitfire.chemistry.analysis`` (plotting / Cantera post-processing only),
* loads the reference's own ``time/*.py``, ``chemistry/library.py``, ``chemistry/reactors.py``,
  ``chemistry/flamelet.py`` and ``chemistry/tabulation.py`` by file path.

``reference_mechanism(path, phase)`` returns an object with the ChemicalMechanismSpec attributes those modules use,
whose ``griffon`` is a reference ``PyCombustionKernels`` filled through the same setter sequence as
``mechanism.py:122-258`` from the project loader's data. Nothing here is imported by the product or by the GPU
tests; it only generates the golden fixtures under ``tests/golden``.
"""

import glob
import importlib.machinery
import importlib.util
import os
import sys
import types

REF_ROOT = os.environ.get('SPITFIRE_REFERENCE')  # the reference checkout (tests/golden/make_golden.py sets it)
HERE = os.path.dirname(os.path.abspath(__file__))


def _ext_path():
    cands = glob.glob(os.path.join(HERE, '_ref', 'griffon*.so'))
    if not cands:
        raise FileNotFoundError('reference Griffon not built: run `make -C oracle ref` where the reference exists')
    return cands[0]


def _load_file(modname, path):
    spec = importlib.util.spec_from_file_location(modname, path)
    mod = importlib.util.module_from_spec(spec)
    sys.modules[modname] = mod
    spec.loader.exec_module(mod)
    return mod


_loaded = {}


def load_reference():
    """Import the reference modules; returns a namespace with griffon, odesolve, HomogeneousReactor, Flamelet, ..."""
    if _loaded:
        return _loaded['ns']
    if not REF_ROOT or not os.path.isdir(os.path.join(REF_ROOT, 'src', 'spitfire')):
        raise FileNotFoundError('set SPITFIRE_REFERENCE to a checkout of the reference Spitfire')
    src = os.path.join(REF_ROOT, 'src', 'spitfire')
    for pkg in ('spitfire', 'spitfire.time', 'spitfire.chemistry', 'spitfire.griffon'):
        m = types.ModuleType(pkg)
        m.__path__ = []
        sys.modules[pkg] = m
    loader = importlib.machinery.ExtensionFileLoader('spitfire.griffon.griffon', _ext_path())
    spec = importlib.util.spec_from_loader('spitfire.griffon.griffon', loader)
    griffon = importlib.util.module_from_spec(spec)
    loader.exec_module(griffon)
    sys.modules['spitfire.griffon.griffon'] = griffon
    if 'matplotlib' not in sys.modules:
        mpl = types.ModuleType('matplotlib')
        plt = types.ModuleType('matplotlib.pyplot')
        mpl.pyplot = plt
        sys.modules['matplotlib'] = mpl
        sys.modules['matplotlib.pyplot'] = plt
    ana = types.ModuleType('spitfire.chemistry.analysis')
    sys.modules['spitfire.chemistry.analysis'] = ana
    mods = {}
    for name in ('stepcontrol', 'methods', 'nonlinear', 'integrator'):
        mods[name] = _load_file('spitfire.time.' + name, os.path.join(src, 'time', name + '.py'))
    for name in ('library', 'reactors', 'flamelet', 'tabulation'):
        mods[name] = _load_file('spitfire.chemistry.' + name, os.path.join(src, 'chemistry', name + '.py'))
    ns = types.SimpleNamespace(griffon=griffon, **mods)
    _loaded['ns'] = ns
    return ns


class ReferenceMechanism:
    """ChemicalMechanismSpec stand-in for the reference modules: project loader data + reference Griffon."""

    def __init__(self, path, phase=None):
        sys.path.insert(0, os.path.dirname(HERE))
        from spitfire_gb300.mechanism import ChemicalMechanismSpec
        ns = load_reference()
        self.spec = ChemicalMechanismSpec(cantera_input=path, group_name=phase) if phase else \
            ChemicalMechanismSpec(cantera_input=path)
        self._griffon = ns.griffon.PyCombustionKernels()
        self.spec._populate_griffon(self._griffon)

    @property
    def griffon(self):
        return self._griffon

    def __getattr__(self, item):
        return getattr(self.spec, item)
