"""GB300-native PandemicThrust daily simulation step.

The compute path is the native library ``_build/libpandemic_gb300.so`` (hand-written
sm_103a CUDA kernels behind the C ABI in ``include/pandemic_gb300.h``).  This module
is a thin ctypes binding with the flow of the reference's ``class PandemicSim``
(PandemicThrust/PandemicThrust/PandemicSim.h:68-281): construct from the
constants.csv parameters and a seed, ``setupSim``, then ``runToCompletion`` or one
day at a time, then the generation counts behind ``output_rn.csv``.

There is no fallback: if the native library is missing or no CUDA device is
available, the calls raise.
"""
import ctypes
import os

import numpy as np

from .build import build as _build, LIB as LIBRARY_PATH, CLI as CLI_PATH, BATCH_CLI as BATCH_CLI_PATH

__all__ = ["PandemicSim", "PandemicBatch", "Params", "Interventions", "load_library", "build", "PtError", "LIBRARY_PATH",
           "CLI_PATH", "BATCH_CLI_PATH", "PT_OK", "PT_DONE", "PT_FINISHED"]

PT_OK, PT_DONE, PT_FINISHED = 0, 1, 2
PT_ERR_ARG, PT_ERR_IO, PT_ERR_PARSE, PT_ERR_OOM, PT_ERR_CUDA, PT_ERR_STATE, PT_ERR_TIMEOUT = -1, -2, -3, -4, -5, -6, -7
_STATUS = {0: "PT_OK", 1: "PT_DONE", 2: "PT_FINISHED", -1: "PT_ERR_ARG", -2: "PT_ERR_IO", -3: "PT_ERR_PARSE",
           -4: "PT_ERR_OOM", -5: "PT_ERR_CUDA", -6: "PT_ERR_STATE", -7: "PT_ERR_TIMEOUT"}


class PtError(RuntimeError):
    def __init__(self, code, message):
        super().__init__("%s: %s" % (_STATUS.get(code, code), message))
        self.code = code


class Params(ctypes.Structure):
    """pt_params: the nine numeric columns of constants.csv, in file order."""
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

    @classmethod
    def from_dict(cls, d):
        p = cls()
        for name, _ in cls._fields_:
            setattr(p, name, d[name])
        return p


class Interventions(ctypes.Structure):
    """pt_interventions: the build's extensions (no reference counterpart); all zero
    reproduces the reference."""
    _fields_ = [
        ("school_closure_start", ctypes.c_int),
        ("school_closure_days", ctypes.c_int),
        ("workplace_absenteeism", ctypes.c_float),
        ("vaccination_coverage", ctypes.c_float),
    ]

    @classmethod
    def from_dict(cls, d):
        iv = cls()
        for name, _ in cls._fields_:
            setattr(iv, name, d.get(name, 0))
        return iv


class Tuning(ctypes.Structure):
    """Launch shapes of the day's kernels (pt_tuning); every choice gives identical results."""
    _fields_ = [("infect_coop", ctypes.c_int), ("infect_blocks_per_sm", ctypes.c_int),
                ("radix_blocks_per_sm", ctypes.c_int), ("sched_tf", ctypes.c_int), ("dense_level", ctypes.c_int),
                ("radix_threads", ctypes.c_int)]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}

    @classmethod
    def from_dict(cls, d):
        t = cls()
        for name, _ in cls._fields_:
            setattr(t, name, int(d[name]))
        return t


class Info(ctypes.Structure):
    _fields_ = [
        ("number_people", ctypes.c_int), ("number_households", ctypes.c_int),
        ("number_workplaces", ctypes.c_int), ("number_adults", ctypes.c_int),
        ("number_children", ctypes.c_int), ("current_day", ctypes.c_int),
        ("days_run", ctypes.c_int), ("infected_count", ctypes.c_int),
        ("rand_offset", ctypes.c_uint64), ("seeds", ctypes.c_int * 4),
        ("type_count", ctypes.c_int * 14), ("type_offset", ctypes.c_int * 14),
        ("infectiousness", ctypes.c_float * 2), ("max_day_of_peak", ctypes.c_int),
        ("max_infected_proportion", ctypes.c_float), ("sm_count", ctypes.c_int),
        ("device_bytes", ctypes.c_uint64), ("bucket_entries_scheduled", ctypes.c_uint64),
        ("bucket_entries_materialised", ctypes.c_uint64),
    ]


EXPORTS = [
    "pt_params_from_csv", "pt_seed_from_file", "pt_create", "pt_setup", "pt_step_day", "pt_run",
    "pt_final_gen_counts", "pt_reset_epidemic", "pt_get_info", "pt_get_person_state",
    "pt_get_population", "pt_get_day_tables", "pt_set_full_tables", "pt_set_timing", "pt_get_stage_ms",
    "pt_get_day_stage_ms", "pt_set_interventions", "pt_batch_set_interventions",
    "pt_launch_count", "pt_transfer_bytes", "pt_destroy", "pt_last_error",
    "pt_batch_create", "pt_batch_setup", "pt_batch_run", "pt_batch_step_day", "pt_batch_reset_epidemic",
    "pt_batch_size", "pt_batch_counts", "pt_batch_final_gen_counts", "pt_batch_get_info",
    "pt_batch_get_person_state", "pt_batch_get_population", "pt_batch_set_timing", "pt_batch_get_stage_ms",
    "pt_batch_transfer_bytes", "pt_batch_destroy", "pt_batch_last_error",
    "pt_set_tuning", "pt_get_tuning", "pt_autotune", "pt_batch_set_tuning", "pt_batch_get_tuning",
    "pt_batch_autotune", "pt_selftest_bounded_wait", "pt_selftest_errand_lookup", "pt_trim_device_memory",
    "pt_bucket_table_static",
]

_lib = None


def build(verbose=False, force=False):
    return _build(verbose=verbose, force=force)


def load_library(path=None):
    """Loads the native library; raises if it is not built."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    path = path or LIBRARY_PATH
    if not os.path.exists(path):
        raise RuntimeError("native library not built: %s (run pandemicthrust_gb300.build())" % path)
    lib = ctypes.CDLL(path)
    vp, ip, i32p = ctypes.c_void_p, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int32)
    u8p = ctypes.POINTER(ctypes.c_uint8)
    lib.pt_params_from_csv.argtypes = [ctypes.c_char_p, ctypes.POINTER(Params)]
    lib.pt_seed_from_file.argtypes = [ctypes.c_char_p, ip]
    lib.pt_create.argtypes = [ctypes.POINTER(Params), ctypes.c_int, vp, ctypes.POINTER(vp)]
    lib.pt_setup.argtypes = [vp]
    lib.pt_step_day.argtypes = [vp, ip, ip]
    lib.pt_run.argtypes = [vp, ip, ip, ip]
    lib.pt_final_gen_counts.argtypes = [vp, ip, ip]
    lib.pt_reset_epidemic.argtypes = [vp]
    lib.pt_get_info.argtypes = [vp, ctypes.POINTER(Info)]
    lib.pt_get_person_state.argtypes = [vp] + [u8p] * 7
    lib.pt_get_population.argtypes = [vp] + [i32p] * 5
    lib.pt_get_day_tables.argtypes = [vp, i32p, i32p, i32p, i32p, ip, ip]
    lib.pt_set_timing.argtypes = [vp, ctypes.c_int]
    lib.pt_set_full_tables.argtypes = [vp, ctypes.c_int]
    lib.pt_get_stage_ms.argtypes = [vp, ctypes.POINTER(ctypes.c_float), ip]
    lib.pt_get_day_stage_ms.argtypes = [vp, ctypes.c_int, ctypes.POINTER(ctypes.c_float)]
    lib.pt_set_interventions.argtypes = [vp, ctypes.POINTER(Interventions)]
    lib.pt_batch_set_interventions.argtypes = [vp, ctypes.POINTER(Interventions)]
    tp = ctypes.POINTER(Tuning)
    for pre in ("pt_", "pt_batch_"):
        getattr(lib, pre + "set_tuning").argtypes = [vp, tp]
        getattr(lib, pre + "get_tuning").argtypes = [vp, tp]
        getattr(lib, pre + "autotune").argtypes = [vp, ctypes.c_int, tp]
    lib.pt_selftest_bounded_wait.argtypes = [ctypes.c_int, ctypes.c_int64, ctypes.POINTER(ctypes.c_uint32)]
    lib.pt_selftest_errand_lookup.argtypes = [ctypes.POINTER(ctypes.c_uint64)]
    lib.pt_trim_device_memory.argtypes = []
    lib.pt_launch_count.restype = ctypes.c_uint64
    lib.pt_launch_count.argtypes = []
    lib.pt_transfer_bytes.argtypes = [vp, ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_uint64)]
    lib.pt_destroy.argtypes = [vp]
    lib.pt_last_error.argtypes = [vp]
    lib.pt_last_error.restype = ctypes.c_char_p
    i64p, u64p = ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_uint64)
    lib.pt_batch_create.argtypes = [ctypes.POINTER(Params), ip, ctypes.c_int, vp, ctypes.POINTER(vp)]
    lib.pt_batch_setup.argtypes = [vp]
    lib.pt_batch_run.argtypes = [vp]
    lib.pt_batch_step_day.argtypes = [vp, ip]
    lib.pt_batch_reset_epidemic.argtypes = [vp]
    lib.pt_batch_size.argtypes = [vp, ip, i64p, i64p]
    lib.pt_batch_counts.argtypes = [vp, ctypes.c_int, ip, ip, ip]
    lib.pt_batch_final_gen_counts.argtypes = [vp, ip, ip]
    lib.pt_batch_get_info.argtypes = [vp, ctypes.c_int, ctypes.POINTER(Info)]
    lib.pt_batch_get_person_state.argtypes = [vp, ctypes.c_int] + [u8p] * 7
    lib.pt_batch_get_population.argtypes = [vp, ctypes.c_int] + [i32p] * 5
    lib.pt_batch_set_timing.argtypes = [vp, ctypes.c_int]
    lib.pt_batch_get_stage_ms.argtypes = [vp, ctypes.POINTER(ctypes.c_float), ip]
    lib.pt_batch_transfer_bytes.argtypes = [vp, u64p, u64p]
    lib.pt_batch_destroy.argtypes = [vp]
    lib.pt_batch_last_error.argtypes = [vp]
    lib.pt_batch_last_error.restype = ctypes.c_char_p
    if path == LIBRARY_PATH:
        _lib = lib
    return lib


def _ptr(a, ctype):
    return a.ctypes.data_as(ctypes.POINTER(ctype)) if a is not None else None


class PandemicSim:
    """One simulation on the current CUDA device (the reference's class PandemicSim)."""

    def __init__(self, params, core_seed, stream=None):
        self.lib = load_library()
        if isinstance(params, dict):
            params = Params.from_dict(params)
        self.params = params
        self.core_seed = int(core_seed)
        h = ctypes.c_void_p()
        rc = self.lib.pt_create(ctypes.byref(params), self.core_seed, stream, ctypes.byref(h))
        if rc != PT_OK:
            raise PtError(rc, self.lib.pt_last_error(None).decode())
        self.h = h

    def _check(self, rc, ok=(PT_OK,)):
        if rc not in ok:
            raise PtError(rc, self.lib.pt_last_error(self.h).decode())
        return rc

    # PandemicSim::setupSim
    def setupSim(self):
        self._check(self.lib.pt_setup(self.h))

    def info(self):
        i = Info()
        self._check(self.lib.pt_get_info(self.h, ctypes.byref(i)))
        return _info_dict(i)

    def step_day(self):
        """One day: returns (status, counts16, infected_count)."""
        c = (ctypes.c_int * 16)()
        n = ctypes.c_int(0)
        rc = self._check(self.lib.pt_step_day(self.h, c, ctypes.byref(n)), ok=(PT_OK, PT_DONE, PT_FINISHED))
        return rc, list(c), n.value

    # PandemicSim::runToCompletion (day loop on the device)
    def runToCompletion(self):
        counts = np.zeros((256, 16), dtype=np.int32)
        infected = np.zeros(256, dtype=np.int32)
        rows = ctypes.c_int(0)
        self._check(self.lib.pt_run(self.h, _ptr(counts, ctypes.c_int), _ptr(infected, ctypes.c_int),
                                    ctypes.byref(rows)))
        return counts[:rows.value].copy(), infected[:rows.value].copy()

    def final_gen_counts(self):
        gp = np.zeros(256, dtype=np.int32)
        gs = np.zeros(256, dtype=np.int32)
        self._check(self.lib.pt_final_gen_counts(self.h, _ptr(gp, ctypes.c_int), _ptr(gs, ctypes.c_int)))
        return gp, gs

    def reset_epidemic(self):
        self._check(self.lib.pt_reset_epidemic(self.h))

    def person_state(self):
        n = self.info()["number_people"]
        out = {k: np.zeros(n, dtype=np.uint8) for k in ("status_p", "status_s", "day_p", "day_s", "gen_p", "gen_s", "age")}
        self._check(self.lib.pt_get_person_state(self.h, *[_ptr(out[k], ctypes.c_uint8) for k in
                                                           ("status_p", "status_s", "day_p", "day_s", "gen_p", "gen_s", "age")]))
        return out

    def population(self):
        i = self.info()
        N, H, L = i["number_people"], i["number_households"], i["number_workplaces"]
        out = dict(household=np.zeros(N, np.int32), household_offset=np.zeros(H + 1, np.int32),
                   workplace=np.zeros(N, np.int32), workplace_people=np.zeros(N, np.int32),
                   workplace_offset=np.zeros(L + 1, np.int32))
        self._check(self.lib.pt_get_population(self.h, *[_ptr(out[k], ctypes.c_int32) for k in
                                                         ("household", "household_offset", "workplace",
                                                          "workplace_people", "workplace_offset")]))
        return out

    def day_tables(self):
        i = self.info()
        N, L = i["number_people"], i["number_workplaces"]
        infected = np.zeros(N, np.int32)
        keys = np.zeros(3 * N, np.int32)
        people = np.zeros(3 * N, np.int32)
        offsets = np.zeros(10 * L + 1, np.int32)
        e, b = ctypes.c_int(0), ctypes.c_int(0)
        self._check(self.lib.pt_get_day_tables(self.h, _ptr(infected, ctypes.c_int32), _ptr(keys, ctypes.c_int32),
                                               _ptr(people, ctypes.c_int32), _ptr(offsets, ctypes.c_int32),
                                               ctypes.byref(e), ctypes.byref(b)))
        return dict(infected=infected, keys=keys[:e.value], people=people[:e.value],
                    offsets=offsets[:b.value + 1], entries=e.value, buckets=b.value)

    def set_interventions(self, iv):
        """School closure, workplace absenteeism, vaccination (a dict or Interventions)."""
        if isinstance(iv, dict):
            iv = Interventions.from_dict(iv)
        self._check(self.lib.pt_set_interventions(self.h, ctypes.byref(iv)))

    def set_full_tables(self, on=True):
        """Materialise every bucket each day (complete tables for day_tables())."""
        self._check(self.lib.pt_set_full_tables(self.h, 1 if on else 0))

    def set_timing(self, on=True):
        self._check(self.lib.pt_set_timing(self.h, 1 if on else 0))

    def set_tuning(self, t):
        """Launch shapes (a dict or Tuning): infect_coop, infect_blocks_per_sm, radix_blocks_per_sm."""
        t = Tuning.from_dict(t) if isinstance(t, dict) else t
        self._check(self.lib.pt_set_tuning(self.h, ctypes.byref(t)))

    def tuning(self):
        t = Tuning()
        self._check(self.lib.pt_get_tuning(self.h, ctypes.byref(t)))
        return t.as_dict()

    def autotune(self, days=0):
        """Times the candidate launch shapes on the first `days` days (0: all), keeps the fastest."""
        t = Tuning()
        self._check(self.lib.pt_autotune(self.h, int(days), ctypes.byref(t)))
        return t.as_dict()

    STAGES = ("sweep", "infected_list", "schedule", "digit_bases", "bucket_sort", "bucket_offsets", "infect", "apply")

    def stage_ms(self):
        """Device ms per stage since the last call: ({weekday: {...}, weekend: {...}}, (weekdays, weekend days))."""
        a = (ctypes.c_float * 16)()
        days = (ctypes.c_int * 2)()
        self._check(self.lib.pt_get_stage_ms(self.h, a, days))
        out = {"weekday": {n: a[k] for k, n in enumerate(self.STAGES)},
               "weekend": {n: a[8 + k] for k, n in enumerate(self.STAGES)}}
        return out, (days[0], days[1])

    def transfer_bytes(self):
        """(host-to-device, device-to-host) bytes this simulation has copied."""
        a, b = ctypes.c_uint64(0), ctypes.c_uint64(0)
        self._check(self.lib.pt_transfer_bytes(self.h, ctypes.byref(a), ctypes.byref(b)))
        return a.value, b.value

    def close(self):
        if getattr(self, "h", None):
            self.lib.pt_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _info_dict(i):
    return {name: (list(getattr(i, name)) if hasattr(getattr(i, name), "__len__") else getattr(i, name))
            for name, _ in Info._fields_}


class PandemicBatch:
    """Many independent simulations advanced together on the current CUDA device.

    Instance k gives exactly what ``PandemicSim(params[k], core_seeds[k])`` gives run
    alone.  The reference runs one process per scenario and seed (its PythonBatcher
    scripts); here every day is one set of launches over all instances and the day
    loop is one CUDA graph.
    """

    def __init__(self, params, core_seeds, stream=None):
        self.lib = load_library()
        params = [Params.from_dict(p) if isinstance(p, dict) else p for p in params]
        if len(params) != len(core_seeds):
            raise ValueError("one core seed per instance")
        self.k = len(params)
        self.params = params
        arr = (Params * self.k)(*params)
        seeds = (ctypes.c_int * self.k)(*[int(x) for x in core_seeds])
        h = ctypes.c_void_p()
        rc = self.lib.pt_batch_create(arr, seeds, self.k, stream, ctypes.byref(h))
        if rc != PT_OK:
            raise PtError(rc, self.lib.pt_batch_last_error(None).decode())
        self.h = h

    def _check(self, rc, ok=(PT_OK,)):
        if rc not in ok:
            raise PtError(rc, self.lib.pt_batch_last_error(self.h).decode())
        return rc

    def setup(self):
        self._check(self.lib.pt_batch_setup(self.h))

    def run(self):
        """Every instance to completion."""
        self._check(self.lib.pt_batch_run(self.h))

    def step_day(self):
        """One day of every running instance: (status, instances still running)."""
        n = ctypes.c_int(0)
        rc = self._check(self.lib.pt_batch_step_day(self.h, ctypes.byref(n)), ok=(PT_OK, PT_DONE, PT_FINISHED))
        return rc, n.value

    def reset_epidemic(self):
        self._check(self.lib.pt_batch_reset_epidemic(self.h))

    def set_interventions(self, ivs):
        """One intervention dict (or Interventions) per instance."""
        arr = (Interventions * self.k)(*[Interventions.from_dict(i) if isinstance(i, dict) else i for i in ivs])
        self._check(self.lib.pt_batch_set_interventions(self.h, arr))

    def size(self):
        """(instances, persons, persons including padding)."""
        k, n, p = ctypes.c_int(0), ctypes.c_int64(0), ctypes.c_int64(0)
        self._check(self.lib.pt_batch_size(self.h, ctypes.byref(k), ctypes.byref(n), ctypes.byref(p)))
        return k.value, n.value, p.value

    def counts(self, k):
        """(counts [days, 16], infected [days]) of instance k, as PandemicSim.runToCompletion."""
        counts = np.zeros((256, 16), dtype=np.int32)
        infected = np.zeros(256, dtype=np.int32)
        rows = ctypes.c_int(0)
        self._check(self.lib.pt_batch_counts(self.h, k, _ptr(counts, ctypes.c_int), _ptr(infected, ctypes.c_int),
                                             ctypes.byref(rows)))
        return counts[:rows.value].copy(), infected[:rows.value].copy()

    def days_run(self):
        """Statistics rows of every instance."""
        out = np.zeros(self.k, dtype=np.int64)
        for k in range(self.k):
            rows = ctypes.c_int(0)
            self._check(self.lib.pt_batch_counts(self.h, k, None, None, ctypes.byref(rows)))
            out[k] = rows.value
        return out

    def final_gen_counts(self):
        """(gen_p, gen_s), each [instances, 256]."""
        gp = np.zeros((self.k, 256), dtype=np.int32)
        gs = np.zeros((self.k, 256), dtype=np.int32)
        self._check(self.lib.pt_batch_final_gen_counts(self.h, _ptr(gp, ctypes.c_int), _ptr(gs, ctypes.c_int)))
        return gp, gs

    def info(self, k):
        i = Info()
        self._check(self.lib.pt_batch_get_info(self.h, k, ctypes.byref(i)))
        return _info_dict(i)

    def person_state(self, k):
        n = self.info(k)["number_people"]
        names = ("status_p", "status_s", "day_p", "day_s", "gen_p", "gen_s", "age")
        out = {name: np.zeros(n, dtype=np.uint8) for name in names}
        self._check(self.lib.pt_batch_get_person_state(self.h, k, *[_ptr(out[name], ctypes.c_uint8) for name in names]))
        return out

    def population(self, k):
        i = self.info(k)
        N, H, L = i["number_people"], i["number_households"], i["number_workplaces"]
        out = dict(household=np.zeros(N, np.int32), household_offset=np.zeros(H + 1, np.int32),
                   workplace=np.zeros(N, np.int32), workplace_people=np.zeros(N, np.int32),
                   workplace_offset=np.zeros(L + 1, np.int32))
        self._check(self.lib.pt_batch_get_population(self.h, k, *[_ptr(out[n], ctypes.c_int32) for n in
                                                                   ("household", "household_offset", "workplace",
                                                                    "workplace_people", "workplace_offset")]))
        return out

    def set_timing(self, on=True):
        self._check(self.lib.pt_batch_set_timing(self.h, 1 if on else 0))

    def set_tuning(self, t):
        t = Tuning.from_dict(t) if isinstance(t, dict) else t
        self._check(self.lib.pt_batch_set_tuning(self.h, ctypes.byref(t)))

    def tuning(self):
        t = Tuning()
        self._check(self.lib.pt_batch_get_tuning(self.h, ctypes.byref(t)))
        return t.as_dict()

    def autotune(self, days=0):
        t = Tuning()
        self._check(self.lib.pt_batch_autotune(self.h, int(days), ctypes.byref(t)))
        return t.as_dict()

    def stage_ms(self):
        a = (ctypes.c_float * 16)()
        days = (ctypes.c_int * 2)()
        self._check(self.lib.pt_batch_get_stage_ms(self.h, a, days))
        out = {"weekday": {n: a[k] for k, n in enumerate(PandemicSim.STAGES)},
               "weekend": {n: a[8 + k] for k, n in enumerate(PandemicSim.STAGES)}}
        return out, (days[0], days[1])

    def transfer_bytes(self):
        a, b = ctypes.c_uint64(0), ctypes.c_uint64(0)
        self._check(self.lib.pt_batch_transfer_bytes(self.h, ctypes.byref(a), ctypes.byref(b)))
        return a.value, b.value

    def close(self):
        if getattr(self, "h", None):
            self.lib.pt_batch_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def launch_count():
    return load_library().pt_launch_count()
