"""ctypes binding of libgpi_fdtd.so (declared in include/gpi_fdtd.h).

This is the same binding a Julia host makes with `ccall`; the Python host
uses it to drive the engine.  Loading fails loudly when the library has not
been built: there is no CPU fallback.
"""
import ctypes
import threading
import os

from . import _build

GPI_OK = 0
STATUS = {0: "GPI_OK", -1: "GPI_E_INVALID", -2: "GPI_E_NOMEM", -3: "GPI_E_CUDA", -4: "GPI_E_UNSUPPORTED",
          -5: "GPI_E_STATE"}
ACOUSTIC, ELASTIC = 0, 1
FORWARD, FORWARD_SAVE, ADJOINT, BORN = 0, 1, 2, 3
FACE = {"zmin": 1, "zmax": 2, "ymin": 4, "ymax": 8, "xmin": 16, "xmax": 32}
FIELD = {"p": 0, "vx": 1, "vy": 2, "vz": 3, "tauxx": 4, "tauyy": 5, "tauzz": 6, "tauxy": 7, "tauxz": 8, "tauyz": 9}

EXPORTS = ["gpi_plan_create", "gpi_plan_destroy", "gpi_last_error", "gpi_set_stream", "gpi_plan_bytes",
           "gpi_set_medium", "gpi_set_pml", "gpi_set_sources", "gpi_clear_sources", "gpi_set_receivers",
           "gpi_run", "gpi_get_records", "gpi_get_gradient", "gpi_get_field", "gpi_last_launches",
           "gpi_set_graph", "gpi_query", "gpi_checkpoint_schedule", "gpi_set_snapshots", "gpi_get_snapshot",
           "gpi_forward_acoustic2d_noalloc", "gpi_set_born", "gpi_plan_estimate", "gpi_server_create",
           "gpi_server_destroy", "gpi_server_submit", "gpi_server_poll", "gpi_server_wait", "gpi_server_records",
           "gpi_server_gradient", "gpi_server_times", "gpi_server_message", "gpi_server_release",
           "gpi_batch_create", "gpi_batch_add", "gpi_batch_advance", "gpi_batch_finished", "gpi_batch_launches",
           "gpi_batch_error", "gpi_batch_destroy", "gpi_set_adjoint_l2", "gpi_set_illum", "gpi_get_illum"]


class PlanDesc(ctypes.Structure):
    _fields_ = [("physics", ctypes.c_int32), ("ndim", ctypes.c_int32), ("order", ctypes.c_int32),
                ("nz", ctypes.c_int32), ("ny", ctypes.c_int32), ("nx", ctypes.c_int32),
                ("npml", ctypes.c_int32), ("nbound", ctypes.c_int32), ("pml_faces", ctypes.c_int32),
                ("rigid_faces", ctypes.c_int32), ("free_faces", ctypes.c_int32), ("nt", ctypes.c_int32),
                ("nshots", ctypes.c_int32), ("npw", ctypes.c_int32), ("checkpoints", ctypes.c_int32),
                ("imaging", ctypes.c_int32), ("reserved", ctypes.c_int32 * 2),
                ("dt", ctypes.c_double), ("dz", ctypes.c_double), ("dy", ctypes.c_double), ("dx", ctypes.c_double)]


class ServerDesc(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int32), ("max_inflight", ctypes.c_int32), ("max_batch", ctypes.c_int32),
                ("reserved", ctypes.c_int32), ("hbm_budget", ctypes.c_size_t)]


class Proj(ctypes.Structure):
    _fields_ = [("shot", ctypes.c_int32), ("field", ctypes.c_int32), ("n", ctypes.c_int32), ("pad", ctypes.c_int32),
                ("colptr", ctypes.c_void_p), ("rowval", ctypes.c_void_p), ("nzval", ctypes.c_void_p),
                ("data", ctypes.c_void_p)]


class Request(ctypes.Structure):
    _fields_ = [("plan", PlanDesc), ("gradient", ctypes.c_int32), ("nsrc", ctypes.c_int32), ("nrec", ctypes.c_int32),
                ("graph", ctypes.c_int32), ("mod", ctypes.c_void_p), ("pml", ctypes.c_void_p),
                ("src", ctypes.POINTER(Proj)), ("rec", ctypes.POINTER(Proj))]


class EngineError(RuntimeError):
    pass


_LIB = None
_LOAD_LOCK = threading.Lock()


def lib_path():
    return _build.LIB


def load():
    """Load the engine; raises if it is missing (build it with _build.build()).
    Thread-safe: plans are created on the serving loop's worker threads."""
    if _LIB is not None:
        return _LIB
    with _LOAD_LOCK:
        return _load()


def _load():
    global _LIB
    if _LIB is not None:
        return _LIB
    path = lib_path()
    if not os.path.exists(path):
        raise EngineError("libgpi_fdtd.so is not built (%s); run __graft_entry__.build() or "
                          "geophyinv_gb300._build.build()" % path)
    L = ctypes.CDLL(path)
    vp, i32, i64p, fp = ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p
    L.gpi_plan_create.argtypes = [ctypes.POINTER(PlanDesc), ctypes.POINTER(ctypes.c_void_p)]
    L.gpi_plan_destroy.argtypes = [vp]
    L.gpi_plan_destroy.restype = None
    L.gpi_last_error.argtypes = [vp]
    L.gpi_last_error.restype = ctypes.c_char_p
    L.gpi_set_stream.argtypes = [vp, vp]
    L.gpi_plan_bytes.argtypes = [vp, ctypes.POINTER(ctypes.c_size_t)]
    L.gpi_set_medium.argtypes = [vp, vp, i32]
    L.gpi_set_born.argtypes = [vp, vp, i32]
    L.gpi_set_pml.argtypes = [vp, i32, i32, fp, fp, fp]
    L.gpi_set_sources.argtypes = [vp, i32, i32, i32, i32, i64p, i64p, fp, fp]
    L.gpi_clear_sources.argtypes = [vp, i32, i32]
    L.gpi_set_receivers.argtypes = [vp, i32, i32, i32, i64p, i64p, fp]
    L.gpi_run.argtypes = [vp, i32]
    L.gpi_get_records.argtypes = [vp, i32, i32, fp, i32]
    L.gpi_get_gradient.argtypes = [vp, i32, fp, i32]
    L.gpi_get_field.argtypes = [vp, i32, i32, i32, fp, i32]
    L.gpi_last_launches.argtypes = [vp, ctypes.POINTER(ctypes.c_int64)]
    L.gpi_set_graph.argtypes = [vp, i32]
    L.gpi_query.argtypes = [vp, ctypes.POINTER(ctypes.c_int32)]
    L.gpi_set_snapshots.argtypes = [vp, i32, i32, ctypes.POINTER(ctypes.c_int32)]
    L.gpi_get_snapshot.argtypes = [vp, i32, i32, i32, fp, i32]
    L.gpi_set_illum.argtypes = [vp, i32]
    L.gpi_get_illum.argtypes = [vp, ctypes.POINTER(ctypes.c_double), i32]
    L.gpi_checkpoint_schedule.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_int64),
                                          ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int32)]
    L.gpi_forward_acoustic2d_noalloc.argtypes = [ctypes.POINTER(PlanDesc), fp, fp, fp, i32, i32, i64p, i64p, fp, fp,
                                                 i32, vp, vp, vp, vp, vp, vp, vp]
    L.gpi_plan_estimate.argtypes = [ctypes.POINTER(PlanDesc), ctypes.POINTER(ctypes.c_size_t)]
    L.gpi_server_create.argtypes = [ctypes.POINTER(ServerDesc), ctypes.POINTER(ctypes.c_void_p)]
    L.gpi_server_destroy.argtypes = [vp]
    L.gpi_server_destroy.restype = None
    L.gpi_server_submit.argtypes = [vp, ctypes.POINTER(Request), ctypes.POINTER(ctypes.c_int64)]
    L.gpi_server_poll.argtypes = [vp, ctypes.c_int64, ctypes.POINTER(ctypes.c_int32)]
    L.gpi_server_wait.argtypes = [vp, ctypes.c_int64]
    L.gpi_server_records.argtypes = [vp, ctypes.c_int64, i32, i32, fp]
    L.gpi_server_gradient.argtypes = [vp, ctypes.c_int64, i32, fp, ctypes.POINTER(ctypes.c_double)]
    L.gpi_server_times.argtypes = [vp, ctypes.c_int64, ctypes.POINTER(ctypes.c_double)]
    L.gpi_server_message.argtypes = [vp, ctypes.c_int64]
    L.gpi_server_message.restype = ctypes.c_char_p
    L.gpi_server_release.argtypes = [vp, ctypes.c_int64]
    L.gpi_set_adjoint_l2.argtypes = [vp, i32, i32, fp, i32, ctypes.POINTER(ctypes.c_double)]
    L.gpi_batch_create.argtypes = [i32, vp, ctypes.POINTER(ctypes.c_void_p)]
    L.gpi_batch_add.argtypes = [vp, vp]
    L.gpi_batch_advance.argtypes = [vp, i32, ctypes.POINTER(ctypes.c_int32)]
    L.gpi_batch_finished.argtypes = [vp, ctypes.POINTER(ctypes.c_void_p), i32, ctypes.POINTER(ctypes.c_int32)]
    L.gpi_batch_launches.argtypes = [vp, ctypes.POINTER(ctypes.c_int64)]
    L.gpi_batch_error.argtypes = [vp]
    L.gpi_batch_error.restype = ctypes.c_char_p
    L.gpi_batch_destroy.argtypes = [vp]
    L.gpi_batch_destroy.restype = None
    _LIB = L
    return L


def check(rc, plan=None):
    if rc != GPI_OK:
        L = load()
        msg = L.gpi_last_error(plan).decode() if True else ""
        raise EngineError("%s: %s" % (STATUS.get(rc, rc), msg))
