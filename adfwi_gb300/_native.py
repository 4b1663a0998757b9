"""ctypes binding of the adfwi_gb300 C ABI (``include/adfwi_gb300.h``).

The library is loaded from ``adfwi_gb300/lib/libadfwi_gb300.so`` (built in-tree by
``adfwi_gb300.build``). There is no fallback: if the library is missing or a call
fails, a RuntimeError says why.
"""
import ctypes
import os

_LIB = None

F32, F64 = 0, 1
SNAP_NATIVE, SNAP_BF16, SNAP_FP16, SNAP_FP24 = 0, 1, 2, 3

c_int32 = ctypes.c_int32
c_int64 = ctypes.c_int64
c_void_p = ctypes.c_void_p


class AcousticDesc(ctypes.Structure):
    _fields_ = [
        ("nz", c_int32), ("nx", c_int32), ("nabc", c_int32), ("free_surface", c_int32),
        ("ns", c_int32), ("nt", c_int32), ("nr", c_int32), ("dtype", c_int32),
        ("checkpoint_segments", c_int32), ("snapshot_every", c_int32),
        ("snapshot_precision", c_int32), ("shots_per_block", c_int32),
        ("dt", ctypes.c_double), ("memory_budget", c_int64), ("ring_depth", c_int32), ("reserved", c_int32),
    ]


class ElasticDesc(ctypes.Structure):
    _fields_ = [
        ("nz", c_int32), ("nx", c_int32), ("nabc", c_int32), ("free_surface", c_int32),
        ("ns", c_int32), ("nt", c_int32), ("nr", c_int32), ("dtype", c_int32),
        ("fd_order", c_int32), ("pml", c_int32), ("checkpoint_segments", c_int32),
        ("snapshot_every", c_int32), ("snapshot_precision", c_int32), ("reserved", c_int32),
        ("dt", ctypes.c_double), ("dx", ctypes.c_double), ("dz", ctypes.c_double),
        ("fdc", ctypes.c_double * 3), ("memory_budget", c_int64),
    ]


class KernelStat(ctypes.Structure):
    _fields_ = [("name", ctypes.c_char * 32), ("launches", c_int64), ("timed_launches", c_int64),
                ("total_ms", ctypes.c_double)]


def library_path():
    return os.path.join(os.path.dirname(os.path.abspath(__file__)), "lib", "libadfwi_gb300.so")


def _bind(lib):
    P = c_void_p
    sig = {
        "adfwi_acoustic_plan_create": (c_int32, [ctypes.POINTER(AcousticDesc), P, P, P, P,
                                                 ctypes.POINTER(c_void_p)]),
        "adfwi_acoustic_plan_destroy": (None, [P]),
        "adfwi_acoustic_plan_create_batched": (c_int32, [ctypes.POINTER(AcousticDesc), P, P, P, P, c_int32, P,
                                                         ctypes.POINTER(c_void_p)]),
        "adfwi_acoustic_plan_models": (c_int32, [P]),
        "adfwi_acoustic_workspace_bytes": (c_int32, [P, c_int32, ctypes.POINTER(c_int64)]),
        "adfwi_acoustic_snapshot_every": (c_int32, [P, ctypes.POINTER(c_int32)]),
        "adfwi_acoustic_forward": (c_int32, [P, P, P, P, P, P, P, P, P, P, P, c_int32, P, c_int64, P]),
        "adfwi_acoustic_backward": (c_int32, [P, P, P, P, P, P, P, P, P, P, P, c_int64, P]),
        "adfwi_acoustic_status": (c_int32, [P, P, c_int64, c_int32, ctypes.POINTER(c_int32), P]),
        "adfwi_acoustic_l2_loss": (c_int32, [P, P, P, ctypes.c_double, c_int32, P, P, c_int64, P]),
        "adfwi_acoustic_l2_sources": (c_int32, [P, P, P, c_int32, P, P, P, c_int64, P]),
        "adfwi_acoustic_backward_l2": (c_int32, [P, P, P, P, c_int32, P, P, P, P, c_int64, P]),
        "adfwi_acoustic_noalloc_status": (c_int32, [P, ctypes.POINTER(c_int32), P]),
        "adfwi_last_error": (c_int32, [ctypes.c_char_p, ctypes.c_size_t]),
        "adfwi_wait_selftest": (c_int32, [c_int64, P, P]),
        "adfwi_profile_start": (c_int32, [c_int32]),
        "adfwi_profile_stop": (c_int32, [ctypes.POINTER(KernelStat), c_int32, ctypes.POINTER(c_int32)]),
        "adfwi_launch_count": (c_int64, []),
        "adfwi_version": (ctypes.c_char_p, []),
    }
    optional = {}
    sig.update({
        "adfwi_elastic_plan_create": (c_int32, [ctypes.POINTER(ElasticDesc), P, P, P, P, P,
                                                ctypes.POINTER(c_void_p)]),
        "adfwi_elastic_plan_destroy": (None, [P]),
        "adfwi_elastic_workspace_bytes": (c_int32, [P, c_int32, ctypes.POINTER(c_int64)]),
        "adfwi_elastic_snapshot_every": (c_int32, [P, ctypes.POINTER(c_int32)]),
        "adfwi_elastic_forward": (c_int32, [P, P, P, P, P, P, c_int32, P, c_int64, P]),
        "adfwi_elastic_backward": (c_int32, [P, P, P, P, P, P, c_int64, P]),
        "adfwi_l2_misfit_workspace_bytes": (c_int32, [c_int32, c_int32, c_int32, ctypes.POINTER(c_int64)]),
        "adfwi_smooth2d_workspace_bytes": (c_int32, [c_int32, c_int32, c_int32, ctypes.POINTER(c_int64)]),
        "adfwi_smooth2d": (c_int32, [c_int32, c_int32, c_int32, P, P, P, c_int64, P]),
        "adfwi_l2_misfit": (c_int32, [c_int32, c_int32, c_int32, c_int32, ctypes.c_double, ctypes.c_double, c_int32,
                                      P, P, P, P, P, c_int64, P]),
    })
    for name, (res, args) in list(sig.items()) + list(optional.items()):
        fn = getattr(lib, name, None)
        if fn is None:
            if name in sig:
                raise RuntimeError("adfwi_gb300 library lacks symbol %s" % name)
            continue
        fn.restype = res
        fn.argtypes = args
    return lib


def lib():
    """The loaded library; raises RuntimeError if it has not been built."""
    global _LIB
    if _LIB is None:
        path = library_path()
        if not os.path.exists(path):
            raise RuntimeError(
                "adfwi_gb300 CUDA library not found at %s; build it with "
                "`python -c 'import __graft_entry__ as g; g.build()'` "
                "(or python -m adfwi_gb300.build)" % path)
        _LIB = _bind(ctypes.CDLL(path))
    return _LIB


def last_error():
    buf = ctypes.create_string_buffer(1024)
    lib().adfwi_last_error(buf, 1024)
    return buf.value.decode(errors="replace")


def check(rc, what):
    if rc != 0:
        raise RuntimeError("%s failed (status %d): %s" % (what, rc, last_error()))


def ptr(t):
    """Raw device/host pointer of a tensor (None -> NULL)."""
    if t is None:
        return None
    return c_void_p(t.data_ptr())


def stream_handle(device):
    import torch
    return c_void_p(torch.cuda.current_stream(device).cuda_stream)


def launch_count():
    """Kernel launches issued by the library so far in this process."""
    return int(lib().adfwi_launch_count())


def profile_start(timed=True):
    check(lib().adfwi_profile_start(int(bool(timed))), "adfwi_profile_start")


def profile_stop():
    """Per-kernel-class {name: (launches, timed_launches, total_ms)} of the session."""
    out = (KernelStat * 16)()
    n = c_int32()
    check(lib().adfwi_profile_stop(out, 16, ctypes.byref(n)), "adfwi_profile_stop")
    return {out[i].name.decode(): (out[i].launches, out[i].timed_launches, out[i].total_ms) for i in range(n.value)}


def wait_selftest(limit_ns, flag, stream=None):
    """Run the bounded-wait self-test: `flag` (a zeroed int32 CUDA tensor of one element) becomes
    1 once a wait that nothing completes has run out after `limit_ns`."""
    st = ctypes.c_void_p(stream) if stream is not None else stream_handle(flag.device)
    check(lib().adfwi_wait_selftest(int(limit_ns), ptr(flag), st), "adfwi_wait_selftest")
