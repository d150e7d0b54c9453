"""Run the reference's OWN time-stepping and tendency code on numpy shims.

Test infrastructure only (see ``oracle/__init__.py``); used by
``tests/golden/make_golden.py`` in an environment that has the fluidsim
0.8.3 sources.  It never runs where those sources are absent.

The following reference files are executed unmodified, loaded with
``importlib`` from ``<reference>/fluidsim/...`` (``fluidsim/__init__.py`` is
bypassed because it needs fluiddyn/h5py/matplotlib, which are absent):

* ``fluidsim/base/time_stepping/base.py``          (loop, CFL, hysteresis)
* ``fluidsim/base/time_stepping/pseudo_spect.py``  (ExactLinearCoefs, RK4, RK2, RK2_trapezoid, Euler)
* ``fluidsim/base/solvers/pseudo_spect.py``        (compute_freq_diss)
* ``fluidsim/base/state.py``                       (StatePseudoSpectral)
* ``fluidsim/base/setofvariables.py``
* ``fluidsim/solvers/ns2d/solver.py``, ``state.py``
* ``fluidsim/solvers/ns3d/solver.py``, ``state.py``, ``time_stepping.py``

Shimmed (written here, not taken from anywhere): ``transonic`` (no-op
``boost``, ``Transonic().is_transpiled == False`` so the pure-Python
branches of the transonic blocks run), ``fluiddyn.util.mpi`` (one rank),
``fluiddyn.calcul.setofvariables.SetOfVariables`` (ndarray subclass),
``fluidfft.fft3d.operators.vector_product``, and the fluidfft operator
object (``oracle.spectral``).  ``fluidsim.base.solvers.base`` and
``fluidsim.operators.operators3d`` are replaced by minimal stand-ins because
they pull in the parameter/IO machinery; the Simul objects are wired by hand
below instead of by ``SimulBase.__init__``.
"""

import ast
import copy
import importlib.util
import random
import sys
import types
from pathlib import Path

import numpy as np

from .spectral import OperNumpy2D, OperNumpy3D


class _Anything:
    """Accepts the transonic type-annotation syntax and ignores it."""

    def __init__(self, *a, **k):
        pass

    def __getitem__(self, item):
        return _Anything()

    def __sub__(self, other):
        return _Anything()

    __add__ = __sub__

    def __call__(self, *a, **k):
        return _Anything()


class _Transonic:
    is_transpiled = False
    is_transpiling = False
    is_compiled = False

    def use_block(self, name):  # pragma: no cover - never reached
        raise RuntimeError("transpiled blocks are not available")


def _boost(obj=None, **kw):
    if obj is None:
        return lambda o: o
    return obj


class SetOfVariables(np.ndarray):
    """Minimal stand-in for ``fluiddyn.calcul.setofvariables.SetOfVariables``."""

    def __new__(cls, keys=None, shape_variable=None, like=None, value=None,
                info=None, dtype=None):
        if like is not None:
            keys = list(like.keys)
            shape_variable = like.shape[1:]
            dtype = like.dtype if dtype is None else dtype
            info = like.info if info is None else info
        obj = np.empty((len(keys),) + tuple(shape_variable), dtype=dtype).view(cls)
        obj.keys = list(keys)
        obj.nvar = len(keys)
        obj.info = info
        if value is not None:
            obj.fill(value)
        return obj

    def __array_finalize__(self, obj):
        if obj is None:
            return
        self.keys = getattr(obj, "keys", None)
        self.nvar = getattr(obj, "nvar", None)
        self.info = getattr(obj, "info", None)

    def get_var(self, key):
        return np.asarray(self)[self.keys.index(key)]

    def set_var(self, key, value):
        np.asarray(self)[self.keys.index(key)] = value

    def initialize(self, value=0):
        self.fill(value)


def vector_product(ax, ay, az, bx, by, bz):
    """Shim for fluidfft's ``vector_product``: ``a x b``."""
    return ay * bz - az * by, az * bx - ax * bz, ax * by - ay * bx


class _Container:
    """Attribute container with the ``_set_attribs`` / ``_set_child`` calls."""

    def __init__(self, **kw):
        self.__dict__.update(kw)

    def _set_attribs(self, d):
        self.__dict__.update(d)

    def _set_child(self, name, attribs=None):
        child = _Container(**(attribs or {}))
        setattr(self, name, child)
        return child

    def __getitem__(self, key):
        return getattr(self, key)


class _OutputStub:
    path_run = "/nonexistent/refshim-run"  # no saved forcing state to resume

    def one_time_step(self):
        pass

    def print_stdout(self, *a, **k):
        pass


_LOADED = {}


def _module(name, path=None, package=False):
    if name in sys.modules and name in _LOADED:
        return sys.modules[name]
    if path is None:
        mod = types.ModuleType(name)
        if package:
            mod.__path__ = []
    else:
        spec = importlib.util.spec_from_file_location(name, str(path))
        mod = importlib.util.module_from_spec(spec)
        sys.modules[name] = mod
        spec.loader.exec_module(mod)
    sys.modules[name] = mod
    _LOADED[name] = mod
    parent, _, child = name.rpartition(".")
    if parent and parent in sys.modules:
        setattr(sys.modules[parent], child, mod)
    return mod


def load_reference(root):
    """Install the shims and load the reference modules; returns a dict."""
    root = Path(root)
    fs = root / "fluidsim"
    if not (fs / "base" / "time_stepping" / "pseudo_spect.py").exists():
        raise FileNotFoundError(f"fluidsim sources not found under {root}")

    tr = _module("transonic")
    tr.boost = _boost
    tr.Transonic = _Transonic
    tr.Type = tr.NDim = _Anything
    tr.Array = tr.Union = _Anything()

    _module("fluiddyn", package=True)
    _module("fluiddyn.util", package=True)
    mpi = _module("fluiddyn.util.mpi")
    mpi.rank, mpi.nb_proc, mpi.comm = 0, 1, None
    mpi.printby0 = print
    _module("fluiddyn.calcul", package=True)
    _module("fluiddyn.calcul.setofvariables").SetOfVariables = SetOfVariables
    _module("fluidfft", package=True)
    _module("fluidfft.fft3d", package=True)
    _module("fluidfft.fft3d.operators").vector_product = vector_product

    for pkg in ("fluidsim", "fluidsim.base", "fluidsim.base.solvers",
                "fluidsim.base.time_stepping", "fluidsim.solvers",
                "fluidsim.solvers.ns2d", "fluidsim.solvers.ns3d",
                "fluidsim.operators"):
        _module(pkg, package=True)

    _module("fluidsim.base.setofvariables", fs / "base" / "setofvariables.py")

    sb = _module("fluidsim.base.solvers.base")

    class InfoSolverBase(_Container):
        pass

    class SimulBase:
        pass

    sb.InfoSolverBase, sb.SimulBase = InfoSolverBase, SimulBase

    op3 = _module("fluidsim.operators.operators3d")

    def dealiasing_variable(ff_fft, where_dealiased):
        ff_fft[np.nonzero(where_dealiased)] = 0.0

    op3.dealiasing_variable = dealiasing_variable

    m = {}
    m["ps_solver"] = _module("fluidsim.base.solvers.pseudo_spect",
                             fs / "base" / "solvers" / "pseudo_spect.py")
    m["ts_base"] = _module("fluidsim.base.time_stepping.base",
                           fs / "base" / "time_stepping" / "base.py")
    m["ts_ps"] = _module("fluidsim.base.time_stepping.pseudo_spect",
                         fs / "base" / "time_stepping" / "pseudo_spect.py")
    m["state"] = _module("fluidsim.base.state", fs / "base" / "state.py")
    m["ns2d_solver"] = _module("fluidsim.solvers.ns2d.solver",
                               fs / "solvers" / "ns2d" / "solver.py")
    m["ns2d_state"] = _module("fluidsim.solvers.ns2d.state",
                              fs / "solvers" / "ns2d" / "state.py")
    m["ns3d_solver"] = _module("fluidsim.solvers.ns3d.solver",
                               fs / "solvers" / "ns3d" / "solver.py")
    m["ns3d_state"] = _module("fluidsim.solvers.ns3d.state",
                              fs / "solvers" / "ns3d" / "state.py")
    m["ns3d_ts"] = _module("fluidsim.solvers.ns3d.time_stepping",
                           fs / "solvers" / "ns3d" / "time_stepping.py")
    _module("fluidsim.solvers.ns2d.strat", package=True)
    m["ns2d_strat_solver"] = _module("fluidsim.solvers.ns2d.strat.solver",
                                     fs / "solvers" / "ns2d" / "strat" / "solver.py")
    m["ns2d_strat_state"] = _module("fluidsim.solvers.ns2d.strat.state",
                                    fs / "solvers" / "ns2d" / "strat" / "state.py")
    m["ns2d_strat_ts"] = _module("fluidsim.solvers.ns2d.strat.time_stepping",
                                 fs / "solvers" / "ns2d" / "strat" / "time_stepping.py")
    _module("fluidsim.solvers.ns2d.bouss", package=True)
    m["ns2d_bouss_solver"] = _module("fluidsim.solvers.ns2d.bouss.solver",
                                     fs / "solvers" / "ns2d" / "bouss" / "solver.py")
    m["ns2d_bouss_state"] = _module("fluidsim.solvers.ns2d.bouss.state",
                                    fs / "solvers" / "ns2d" / "bouss" / "state.py")
    _module("fluidsim.solvers.ns3d.strat", package=True)
    m["ns3d_strat_solver"] = _module("fluidsim.solvers.ns3d.strat.solver",
                                     fs / "solvers" / "ns3d" / "strat" / "solver.py")
    m["ns3d_strat_state"] = _module("fluidsim.solvers.ns3d.strat.state",
                                    fs / "solvers" / "ns3d" / "strat" / "state.py")
    _module("fluidsim.solvers.ns3d.bouss", package=True)
    m["ns3d_bouss_solver"] = _module("fluidsim.solvers.ns3d.bouss.solver",
                                     fs / "solvers" / "ns3d" / "bouss" / "solver.py")

    # the reference's toroidal / poloidal projectors (methods of its
    # OperatorsPseudoSpectral3D, whose module needs fluidfft): their function
    # definitions are taken from operators3d.py as written and bound to the
    # numpy operator by make_ns3d
    ops_path = fs / "operators" / "operators3d.py"
    for name in ("project_toroidal", "project_poloidal"):
        m[name] = _reference_method(ops_path, "OperatorsPseudoSpectral3D", name)
    # the random phase pairs of the *_phaseshift_random schemes (they draw
    # with the global `random` module, so random.seed makes them repeatable)
    m["get_phases_random_3d"] = _reference_method(ops_path, "OperatorsPseudoSpectral3D",
                                                  "get_phases_random")
    m["get_phases_random_2d"] = _reference_method(
        fs / "operators" / "operators2d.py", "OperatorsPseudoSpectral2D", "get_phases_random")

    # forcing: the reference's forcing makers (specific.py) with
    # fluiddyn's fftw_grid_size raising ImportError, the path a fluidsim
    # installation without pulp (not among fluidsim's dependencies) takes;
    # the coarse-grid methods of its OperatorsPseudoSpectral3D are compiled
    # from operators3d.py as written and bound to the numpy operator
    def fftw_grid_size(nk_min, bases=None, debug=False):
        raise ImportError("pulp is not installed")

    _module("fluiddyn.calcul.easypyfft").fftw_grid_size = fftw_grid_size
    _module("fluidsim.base.forcing", package=True)
    m["forcing_specific"] = _module("fluidsim.base.forcing.specific",
                                    fs / "base" / "forcing" / "specific.py")
    glob = {"nb_proc": 1, "rank": 0,
            "_ik_from_ikc": _reference_function(ops_path, "_ik_from_ikc")}
    for name in ("project_fft_on_realX", "coarse_seq_from_fft_loc",
                 "put_coarse_array_in_array_fft"):
        m[name] = _reference_method(ops_path, "OperatorsPseudoSpectral3D", name, glob)

    # turbulence model: the reference's Smagorinsky + stress tensor, with the
    # SimulExtender plumbing of turb_model/base.py replaced by a stand-in
    _module("fluidsim.base.turb_model", package=True)
    tb = _module("fluidsim.base.turb_model.base")

    class SpecificTurbModelSpectral:
        def __init__(self, sim):
            self.sim = sim
            self.forcing_fft = SetOfVariables(like=sim.state.state_spect,
                                              info="forcing_fft", value=0.0)

    tb.SpecificTurbModelSpectral = SpecificTurbModelSpectral
    m["stress_tensor"] = _module("fluidsim.base.turb_model.stress_tensor",
                                 fs / "base" / "turb_model" / "stress_tensor.py")
    m["smagorinsky"] = _module("fluidsim.base.turb_model.smagorinsky",
                               fs / "base" / "turb_model" / "smagorinsky.py")
    return m


def _compile_def(path, node, extra=None):
    node.decorator_list = []
    mod = ast.Module(body=[node], type_ignores=[])
    ns = {"np": np, "Ac": object, "Af": object, "uniform": random.uniform}
    ns.update(extra or {})
    exec(compile(mod, str(path), "exec"), ns)
    return ns[node.name]


def _reference_method(path, class_name, name, extra=None):
    """Function object of method ``name`` of class ``class_name`` in the
    reference source file ``path``, compiled from that file (decorators such
    as transonic's ``boost`` dropped, annotations resolved to placeholders,
    module globals it reads given in ``extra``)."""
    tree = ast.parse(Path(path).read_text(), filename=str(path))
    for node in tree.body:
        if isinstance(node, ast.ClassDef) and node.name == class_name:
            for item in node.body:
                if isinstance(item, ast.FunctionDef) and item.name == name:
                    return _compile_def(path, item, extra)
    raise LookupError(f"{class_name}.{name} not found in {path}")


def _reference_function(path, name, extra=None):
    """Module-level function ``name`` of the reference source file ``path``."""
    tree = ast.parse(Path(path).read_text(), filename=str(path))
    for node in tree.body:
        if isinstance(node, ast.FunctionDef) and node.name == name:
            return _compile_def(path, node, extra)
    raise LookupError(f"{name} not found in {path}")


def _params(nu_2, nu_4, nu_8, nu_m4, USE_CFL, deltat0, deltat_max, cfl_coef,
            extra, type_time_scheme="RK4"):
    p = _Container(nu_2=nu_2, nu_4=nu_4, nu_8=nu_8, nu_m4=nu_m4)
    p.__dict__.update(extra)
    p.forcing = _Container(enable=False)
    p.time_stepping = _Container(
        USE_T_END=False, t_end=10.0, it_end=10, USE_CFL=USE_CFL,
        type_time_scheme=type_time_scheme, deltat0=deltat0, deltat_max=deltat_max,
        cfl_coef=cfl_coef, max_elapsed=None,
        phaseshift_random=_Container(nb_pairs=1, nb_steps_compute_new_pair=None),
    )
    return p


def make_ns2d(mods, oper: OperNumpy2D, nu_2=0.0, nu_4=0.0, nu_8=0.0,
              nu_m4=0.0, beta=0.0, USE_CFL=False, deltat0=0.2,
              deltat_max=0.2, cfl_coef=None, type_time_scheme="RK4", N=None,
              bouss=False):
    """A reference ns2d ``Simul`` wired around ``oper`` (with ``N`` given:
    the ns2d.strat ``Simul``, ``StateNS2DStrat`` and its time stepping; with
    ``bouss``: the ns2d.bouss ``Simul`` and ``StateNS2DBouss``)."""
    strat = N is not None
    if bouss:
        Simul = mods["ns2d_bouss_solver"].Simul
        State = mods["ns2d_bouss_state"].StateNS2DBouss
    else:
        Simul = (mods["ns2d_strat_solver"] if strat else mods["ns2d_solver"]).Simul
        State = (mods["ns2d_strat_state"].StateNS2DStrat if strat
                 else mods["ns2d_state"].StateNS2D)
    sim = object.__new__(Simul)
    extra = {"beta": beta}
    if strat:
        extra["N"] = N
    sim.params = _params(nu_2, nu_4, nu_8, nu_m4, USE_CFL, deltat0,
                         deltat_max, cfl_coef, extra, type_time_scheme)
    sim.params.time_stepping.cfl_coef_group = None
    if type_time_scheme.endswith("_random"):
        oper = copy.copy(oper)
        oper.get_phases_random = types.MethodType(mods["get_phases_random_2d"], oper)
    info = _Container(solver=_Container(classes=_Container(State=_Container())))
    State._complete_info_solver(info.solver)
    sim.info = info
    sim.oper = oper
    sim.output = _OutputStub()
    sim.is_forcing_enabled = False
    sim.state = State(sim)
    sim.state.state_spect[:] = 0.0
    sim.state.state_phys[:] = 0.0
    if strat:
        sim.time_stepping = mods["ns2d_strat_ts"].TimeSteppingPseudoSpectralStrat(sim)
    else:
        sim.time_stepping = mods["ts_ps"].TimeSteppingPseudoSpectral(sim)
    return sim


class _ForcingStandIn:
    """``sim.forcing`` (``fluidsim/base/forcing/base.py:143-150,194-195``):
    ``compute()`` at most once per time, ``get_forcing()`` the maker's
    ``forcing_fft``."""

    def __init__(self, sim, maker):
        self.sim = sim
        self.forcing_maker = maker
        self._t_last_computed = -np.inf

    def compute(self):
        time = self.sim.time_stepping.t
        if time > self._t_last_computed:
            self.forcing_maker.compute()
            self._t_last_computed = time

    def get_forcing(self):
        return self.forcing_maker.forcing_fft


def _params_oper_class(mods):
    """The numpy operator constructed from ``params`` as fluidsim constructs
    its operators (the forcing makers build their coarse operator with
    ``sim.oper.__class__(params=...)``), carrying the reference's coarse-grid
    methods and fluidfft's ``deltak`` (the largest deltak_i)."""

    class OperNumpy3DFromParams(OperNumpy3D):
        def __init__(self, params):
            po = params.oper
            super().__init__(po.nx, po.ny, po.nz, po.Lx, po.Ly, po.Lz,
                             coef_dealiasing=po.coef_dealiasing)
            self.deltak = max(self.deltakx, self.deltaky, self.deltakz)

    for name in ("project_fft_on_realX", "coarse_seq_from_fft_loc",
                 "put_coarse_array_in_array_fft"):
        setattr(OperNumpy3DFromParams, name, mods[name])
    return OperNumpy3DFromParams


_FORCING_CLASSES = {"tcrandom": "TimeCorrelatedRandomPseudoSpectral",
                    "random": "RandomSimplePseudoSpectral", "proportional": "Proportional"}


def make_ns3d(mods, oper: OperNumpy3D, nu_2=0.0, nu_4=0.0, nu_8=0.0,
              nu_m4=0.0, f=None, USE_CFL=False, deltat0=0.2, deltat_max=0.2,
              cfl_coef=None, smagorinsky_C=None, type_time_scheme="RK4",
              projection=None, no_vz_kz0=False, N=None, bouss=False, forcing=None):
    """A reference ns3d ``Simul`` wired around ``oper`` (with ``N`` given:
    the ns3d.strat ``Simul`` and ``StateNS3DStrat``; with ``bouss`` as well:
    the ns3d.bouss ``Simul``, whose tendencies do not use N).  ``forcing``:
    a dict (type, key_forced, nkmin_forcing, nkmax_forcing, forcing_rate,
    time_correlation, which_root, only_positive) for the reference's own
    forcing maker of that type, created after the time stepping (it reads
    ``time_stepping.t``) and drawing from the global ``np.random``."""
    strat = N is not None
    Simul = (mods["ns3d_bouss_solver"] if bouss else
             mods["ns3d_strat_solver"] if strat else mods["ns3d_solver"]).Simul
    State = mods["ns3d_strat_state"].StateNS3DStrat if strat else mods["ns3d_state"].StateNS3D
    sim = object.__new__(Simul)
    extra = {"f": f, "no_vz_kz0": no_vz_kz0, "projection": projection}
    if strat:
        extra["N"] = N
    sim.params = _params(nu_2, nu_4, nu_8, nu_m4, USE_CFL, deltat0,
                         deltat_max, cfl_coef, extra, type_time_scheme)
    if forcing is not None:
        sim.params.oper = _Container(
            nx=oper.nx, ny=oper.ny, nz=oper.nz, Lx=oper.Lx, Ly=oper.Ly, Lz=oper.Lz,
            type_fft="default", coef_dealiasing=oper.coef_dealiasing)
        sim.params.output = _Container(HAS_TO_SAVE=False)
        fc = forcing
        sim.params.forcing = _Container(
            enable=True, type=fc["type"], key_forced=fc["key_forced"],
            nkmin_forcing=fc["nkmin_forcing"], nkmax_forcing=fc["nkmax_forcing"],
            forcing_rate=fc["forcing_rate"],
            normalized=_Container(type="2nd_degree_eq",
                                  which_root=fc.get("which_root", "minabs"),
                                  constant_rate_of=None),
            random=_Container(only_positive=fc.get("only_positive", False)),
            tcrandom=_Container(time_correlation=fc.get("time_correlation",
                                                        "based_on_forcing_rate")))
        oper = _params_oper_class(mods)(sim.params)
    if projection is not None or type_time_scheme.endswith("_random"):
        oper = copy.copy(oper)
        for name in ("project_toroidal", "project_poloidal"):
            setattr(oper, name, types.MethodType(mods[name], oper))
        oper.get_phases_random = types.MethodType(mods["get_phases_random_3d"], oper)
    info = _Container(solver=_Container(classes=_Container(State=_Container())))
    State._complete_info_solver(info.solver)
    sim.info = info
    sim.oper = oper
    sim.output = _OutputStub()
    sim.is_forcing_enabled = False
    sim.state = State(sim)
    sim.state.state_spect[:] = 0.0
    sim.state.state_phys[:] = 0.0
    sim._init_projection()
    if smagorinsky_C is not None:
        sim.params.oper = _Container(Lx=oper.Lx, nx=oper.nx)
        sim.params.turb_model = _Container(
            enable=True, type="smagorinsky",
            smagorinsky=_Container(C=smagorinsky_C))
        sim.is_turb_model_enabled = True
        sim.turb_model = mods["smagorinsky"].SmagorinskyModel(sim)
    sim.time_stepping = mods["ns3d_ts"].TimeSteppingPseudoSpectralNS3D(sim)
    if forcing is not None:
        Maker = getattr(mods["forcing_specific"], _FORCING_CLASSES[forcing["type"]])
        sim.forcing = _ForcingStandIn(sim, Maker(sim))
        sim.is_forcing_enabled = True
    return sim
