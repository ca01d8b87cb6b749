"""ctypes bindings for the CPU oracle and the reference-derived checker (test infrastructure).

``Oracle`` wraps ``oracle/_build/libptoracle.so`` (the C restatement, pt_oracle.c).
``RefSim`` wraps ``oracle/_ref/libptref.so`` (the reference's own kernels compiled for
the host by build_ref.py); it exists only where the reference tree was present at
build time.  Neither is part of the product: only tests, the smoke entry point and
the benchmark's CPU-baseline leg use this module.
"""
import ctypes
import os
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "libptoracle.so")
REF_SO = os.path.join(HERE, "_ref", "libptref.so")


class PtorParams(ctypes.Structure):
    _fields_ = [
        ("max_days", ctypes.c_int),
        ("r_pandemic", ctypes.c_float),
        ("r_seasonal", ctypes.c_float),
        ("initial_pandemic", ctypes.c_int),
        ("initial_seasonal", ctypes.c_int),
        ("people_scaling", ctypes.c_float),
        ("location_scaling", ctypes.c_float),
        ("percent_symptomatic", ctypes.c_float),
        ("asymp_factor", ctypes.c_float),
    ]


_u8p = ctypes.POINTER(ctypes.c_uint8)
_i32p = ctypes.POINTER(ctypes.c_int32)


class PtorView(ctypes.Structure):
    _fields_ = [
        ("N", ctypes.c_int), ("H", ctypes.c_int), ("L", ctypes.c_int),
        ("adults", ctypes.c_int), ("children", ctypes.c_int),
        ("infected_count", ctypes.c_int), ("current_day", ctypes.c_int),
        ("rand_offset", ctypes.c_uint64),
        ("workplace_rand_offset", ctypes.c_uint64),
        ("errand_rand_offset", ctypes.c_uint64),
        ("seeds", ctypes.c_int * 4),
        ("type_count", ctypes.c_int * 14),
        ("type_offset", ctypes.c_int * 14),
        ("infectiousness", ctypes.c_float * 2),
        ("shedding", (ctypes.c_float * 10) * 6),
        ("status_p", _u8p), ("status_s", _u8p), ("day_p", _u8p), ("day_s", _u8p),
        ("gen_p", _u8p), ("gen_s", _u8p), ("age", _u8p),
        ("household", _i32p), ("household_offset", _i32p), ("workplace", _i32p),
        ("workplace_people", _i32p), ("workplace_offset", _i32p), ("infected", _i32p),
        ("errand_keys", _i32p), ("errand_people", _i32p), ("errand_offset", _i32p),
        ("errand_entries", ctypes.c_int), ("errand_buckets", ctypes.c_int),
    ]


# The default scenario of the reference's constants.csv (PandemicThrust/PandemicThrust/constants.csv:2).
DEFAULT_PARAMS = dict(max_days=100, r_pandemic=1.8, r_seasonal=1.3, initial_pandemic=30,
                      initial_seasonal=30, people_scaling=1.0, location_scaling=1.0,
                      percent_symptomatic=1.0, asymp_factor=0.0)

PARAM_ORDER = ["max_days", "r_pandemic", "r_seasonal", "initial_pandemic", "initial_seasonal",
               "people_scaling", "location_scaling", "percent_symptomatic", "asymp_factor"]


def make_params(**kw):
    d = dict(DEFAULT_PARAMS)
    d.update(kw)
    return d


def params_struct(d):
    p = PtorParams()
    for k in PARAM_ORDER:
        setattr(p, k, d[k])
    return p


def constants_csv_text(d):
    """The constants.csv layout the reference parses (PandemicSim.cu:299-309)."""
    header = "constants," + ",".join([
        "max_days", "reproduction_number_pandemic", "reproduction_number_seasonal",
        "initial_infected_pandemic", "initial_infected_seasonal", "people_scaling_factor",
        "location_scaling_factor", "percent_symptomatic", "asymp_factor"])
    vals = []
    for k in PARAM_ORDER:
        v = d[k]
        if k in ("max_days", "initial_pandemic", "initial_seasonal"):
            vals.append("%d" % int(v))
        else:
            vals.append("%.9g" % float(np.float32(v)))
    return header + "\n" + "constants," + ",".join(vals) + "\n"


def write_inputs(dirpath, d, seed):
    with open(os.path.join(dirpath, "constants.csv"), "w") as fh:
        fh.write(constants_csv_text(d))
    with open(os.path.join(dirpath, "seed.txt"), "w") as fh:
        fh.write("%d\n" % seed)


def _arr(ptr, n, dtype):
    if n <= 0 or not ptr:
        return np.zeros(0, dtype=dtype)
    return np.ctypeslib.as_array(ptr, shape=(n,)).astype(dtype, copy=True)


def view_to_dict(v):
    N, H, L = v.N, v.H, v.L
    nb = v.errand_buckets
    out = dict(
        N=N, H=H, L=L, adults=v.adults, children=v.children,
        infected_count=v.infected_count, current_day=v.current_day,
        rand_offset=v.rand_offset, workplace_rand_offset=v.workplace_rand_offset,
        errand_rand_offset=v.errand_rand_offset, seeds=list(v.seeds),
        type_count=list(v.type_count), type_offset=list(v.type_offset),
        infectiousness=np.array(list(v.infectiousness), dtype=np.float32),
        shedding=np.array([list(r) for r in v.shedding], dtype=np.float32),
        status_p=_arr(v.status_p, N, np.uint8), status_s=_arr(v.status_s, N, np.uint8),
        day_p=_arr(v.day_p, N, np.uint8), day_s=_arr(v.day_s, N, np.uint8),
        gen_p=_arr(v.gen_p, N, np.uint8), gen_s=_arr(v.gen_s, N, np.uint8),
        age=_arr(v.age, N, np.uint8), household=_arr(v.household, N, np.int32),
        household_offset=_arr(v.household_offset, H + 1, np.int32),
        workplace=_arr(v.workplace, N, np.int32),
        workplace_people=_arr(v.workplace_people, N, np.int32),
        workplace_offset=_arr(v.workplace_offset, L + 1, np.int32),
        infected=_arr(v.infected, v.infected_count, np.int32),
        errand_entries=v.errand_entries, errand_buckets=nb,
        errand_keys=_arr(v.errand_keys, v.errand_entries, np.int32),
        errand_people=_arr(v.errand_people, v.errand_entries, np.int32),
        errand_offset=_arr(v.errand_offset, nb + 1 if nb else 0, np.int32),
    )
    return out


_oracle_lib = None


def oracle_lib():
    global _oracle_lib
    if _oracle_lib is None:
        if not os.path.exists(ORACLE_SO):
            from . import build_oracle  # noqa: F401  (sibling build recipe)
            build_oracle.build()
        lib = ctypes.CDLL(ORACLE_SO)
        lib.ptor_create.restype = ctypes.c_void_p
        lib.ptor_create.argtypes = [ctypes.POINTER(PtorParams), ctypes.c_int]
        lib.ptor_destroy.argtypes = [ctypes.c_void_p]
        lib.ptor_setup.argtypes = [ctypes.c_void_p]
        lib.ptor_step_day.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)]
        lib.ptor_count_and_recover.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int)]
        lib.ptor_build_infected.argtypes = [ctypes.c_void_p]
        lib.ptor_build_schedule.argtypes = [ctypes.c_void_p]
        lib.ptor_infect.argtypes = [ctypes.c_void_p]
        lib.ptor_finish_day.argtypes = [ctypes.c_void_p]
        lib.ptor_gen_counts.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)]
        lib.ptor_get_view.argtypes = [ctypes.c_void_p, ctypes.POINTER(PtorView)]
        lib.ptor_run_to_files.argtypes = [ctypes.POINTER(PtorParams), ctypes.c_int, ctypes.c_char_p]
        lib.ptor_recalc_workplace.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int]
        lib.ptor_recalc_weekday_errands.argtypes = [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_int, ctypes.c_int,
                                                    ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)]
        lib.ptor_recalc_weekend_errands.argtypes = [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_int,
                                                    ctypes.POINTER(ctypes.c_int)]
        lib.ptor_threefry2x64.argtypes = [ctypes.POINTER(ctypes.c_uint64)] * 3
        lib.ptor_threefry2x32.argtypes = [ctypes.POINTER(ctypes.c_uint32)] * 3
        lib.ptor_glibc_srand.argtypes = [ctypes.c_void_p, ctypes.c_uint]
        lib.ptor_glibc_rand_next.argtypes = [ctypes.c_void_p]
        lib.ptor_set_threads.argtypes = [ctypes.c_int]
        lib.ptor_set_interventions.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_float,
                                               ctypes.c_float]
        _oracle_lib = lib
    return _oracle_lib


def threefry2x64(ctr, key):
    lib = oracle_lib()
    c = (ctypes.c_uint64 * 2)(*ctr)
    k = (ctypes.c_uint64 * 2)(*key)
    o = (ctypes.c_uint64 * 2)()
    lib.ptor_threefry2x64(c, k, o)
    return [o[0], o[1]]


def threefry2x32(ctr, key):
    lib = oracle_lib()
    c = (ctypes.c_uint32 * 2)(*ctr)
    k = (ctypes.c_uint32 * 2)(*key)
    o = (ctypes.c_uint32 * 2)()
    lib.ptor_threefry2x32(c, k, o)
    return [o[0], o[1]]


def glibc_rand(seed, n):
    lib = oracle_lib()
    st = ctypes.create_string_buffer(34 * 4 + 16)
    lib.ptor_glibc_srand(st, seed & 0xFFFFFFFF)
    return [lib.ptor_glibc_rand_next(st) for _ in range(n)]


class Oracle:
    """The C restatement, stepped day by day."""

    def __init__(self, params, seed, threads=1):
        self.lib = oracle_lib()
        self.lib.ptor_set_threads(threads)
        self.params = dict(params)
        self._p = params_struct(params)
        self.h = self.lib.ptor_create(ctypes.byref(self._p), seed)
        if not self.h:
            raise ValueError("oracle rejected the parameters")

    def set_interventions(self, school_closure_start=0, school_closure_days=0, workplace_absenteeism=0.0,
                          vaccination_coverage=0.0):
        """The build's intervention extensions (no reference counterpart); before setup()."""
        self.lib.ptor_set_interventions(self.h, int(school_closure_start), int(school_closure_days),
                                        float(workplace_absenteeism), float(vaccination_coverage))

    def setup(self):
        rc = self.lib.ptor_setup(self.h)
        if rc != 0:
            raise RuntimeError("oracle setup failed")

    def step_day(self):
        c = (ctypes.c_int * 16)()
        i = ctypes.c_int(0)
        rc = self.lib.ptor_step_day(self.h, c, ctypes.byref(i))
        return rc, list(c), i.value

    def view(self):
        v = PtorView()
        self.lib.ptor_get_view(self.h, ctypes.byref(v))
        return view_to_dict(v)

    def gen_counts(self):
        gp = (ctypes.c_int * 256)()
        gs = (ctypes.c_int * 256)()
        self.lib.ptor_gen_counts(self.h, gp, gs)
        return np.array(list(gp)), np.array(list(gs))

    def close(self):
        if self.h:
            self.lib.ptor_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def oracle_run_to_files(params, seed, dirpath):
    lib = oracle_lib()
    p = params_struct(params)
    return lib.ptor_run_to_files(ctypes.byref(p), seed, dirpath.encode())


_ref_lib = None


def ref_available():
    return os.path.exists(REF_SO)


def ref_lib():
    global _ref_lib
    if _ref_lib is None:
        lib = ctypes.CDLL(REF_SO)
        lib.ptref_create.argtypes = [ctypes.c_char_p]
        lib.ptref_step_day.argtypes = [ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)]
        lib.ptref_get_view.argtypes = [ctypes.POINTER(PtorView)]
        lib.ptref_gen_counts.argtypes = [ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)]
        lib.ptref_threefry2x64.argtypes = [ctypes.POINTER(ctypes.c_uint64)] * 3
        lib.ptref_threefry2x32.argtypes = [ctypes.POINTER(ctypes.c_uint32)] * 3
        lib.ptref_libc_rand.argtypes = [ctypes.c_uint, ctypes.c_int, ctypes.POINTER(ctypes.c_int)]
        lib.ptref_host_recalc_workplace.argtypes = [ctypes.c_int, ctypes.c_int]
        lib.ptref_host_recalc_weekday.argtypes = [ctypes.c_uint64, ctypes.c_int, ctypes.c_int,
                                                  ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)]
        lib.ptref_host_recalc_weekend.argtypes = [ctypes.c_uint64, ctypes.c_int, ctypes.POINTER(ctypes.c_int)]
        _ref_lib = lib
    return _ref_lib


class RefSim:
    """The reference's kernels run on the host (one simulation per process at a time)."""

    def __init__(self, params, seed):
        self.lib = ref_lib()
        self._tmp = tempfile.TemporaryDirectory()
        write_inputs(self._tmp.name, params, seed)
        if self.lib.ptref_create(self._tmp.name.encode()) != 0:
            raise RuntimeError("reference harness failed to load inputs")

    def setup(self):
        if self.lib.ptref_setup() != 0:
            raise RuntimeError("reference harness setup failed")

    def step_day(self):
        c = (ctypes.c_int * 16)()
        i = ctypes.c_int(0)
        rc = self.lib.ptref_step_day(c, ctypes.byref(i))
        return rc, list(c), i.value

    def view(self):
        v = PtorView()
        self.lib.ptref_get_view(ctypes.byref(v))
        return view_to_dict(v)

    def gen_counts(self):
        gp = (ctypes.c_int * 256)()
        gs = (ctypes.c_int * 256)()
        self.lib.ptref_gen_counts(gp, gs)
        return np.array(list(gp)), np.array(list(gs))

    def close(self):
        self.lib.ptref_destroy()
        self._tmp.cleanup()
