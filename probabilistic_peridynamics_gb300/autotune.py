"""Kernel-variant autotuner.

Times each candidate launch configuration of a kernel on the problem it will
run (CUDA events on the integrator's stream) and keeps the fastest.  The
candidates run on scratch copies of every array the step writes, so tuning
never changes the simulation state.  Results are cached per process by a
problem key.
"""
import ctypes

from . import _lib
from ._lib import check, lib

_cache = {}


def time_launches(launch, stream, warmup=3, reps=10):
    """Mean milliseconds of ``launch()`` over ``reps`` launches."""
    import torch
    for _ in range(warmup):
        launch()
    start = torch.cuda.Event(enable_timing=True)
    stop = torch.cuda.Event(enable_timing=True)
    start.record(stream)
    for _ in range(reps):
        launch()
    stop.record(stream)
    stop.synchronize()
    return start.elapsed_time(stop) / reps


#: FusedArgs fields a mixed-precision step writes.
_MIXED_WRITES = ("nlist", "regimes", "vel", "acc", "frc", "n_neigh", "umax",
                 "status")


def _time_layout(integ, tiled, warmup, reps):
    """Milliseconds per step of every tile shape of one layout (tiled or
    untiled), each on scratch copies of the arrays the step writes; the
    untiled kernel of an integrator set up tiled runs on a scratch state
    packed in the reference node order."""
    import torch
    fa = integ._fargs
    tiling = integ.tiling
    scratch = _lib.FusedArgs()
    ctypes.pointer(scratch)[0] = fa  # copy all fields
    keep = []

    def clone(ptr_value, tensor):
        if not ptr_value or tensor is None:
            return ptr_value
        t = tensor.clone()
        keep.append(t)
        return t.data_ptr()

    def fresh(shape, dtype):
        t = torch.empty(shape, dtype=dtype, device=integ.context.device)
        keep.append(t)
        return t.data_ptr()

    tensors = {"nlist": integ.nlist_d, "regimes": integ.regimes_d,
               "vel": integ.vel_d, "acc": integ.acc_d, "frc": integ.frc_d,
               "n_neigh": integ.n_neigh_d, "umax": integ.umax_d,
               "status": integ.status_d}
    for name in _MIXED_WRITES:
        setattr(scratch, name, clone(getattr(scratch, name), tensors[name]))
    for k in range(2):
        scratch.rec[k] = clone(scratch.rec[k], integ.rec_d[k])
        scratch.ulo[k] = clone(scratch.ulo[k], integ.ulo_d[k])
    if tiled:
        # the tiled step writes entries (breaks), regimes, the intact
        # counts and the scheduler words of its tiling
        st = _lib.Tiling()
        ctypes.pointer(st)[0] = tiling.struct
        st.entry = clone(st.entry, tiling.entry_d)
        st.regime = clone(st.regime, tiling.regime_d)
        st.n_neigh = clone(st.n_neigh, tiling.n_neigh_d)
        st.sched = clone(st.sched, tiling.sched_d)
        keep.append(st)
        scratch.tiling = ctypes.addressof(st)
    elif fa.tiling:
        n, mn = integ.nnodes, integ.max_neighbours
        scratch.tiling = None
        scratch.nflags = fresh((n,), torch.int32)
        if scratch.vel:
            scratch.rho32 = fresh((n, 4), torch.float32)
        if scratch.stiffness_corrections:
            scratch.sc32 = fresh((n, mn), torch.float32)
        check(lib().pp_mixed_pack(ctypes.byref(scratch), integ._parity,
                                  integ._stream), "pp_mixed_pack")
    results = {}
    stream = integ.context.stream
    name = "tiled" if tiled else "untiled"
    for variant in range(_lib.PP_MIXED_VARIANTS):
        scratch.variant = variant
        parity = [integ._parity]

        def launch():
            check(lib().pp_fused_step(ctypes.byref(scratch), parity[0],
                                      0.0, 0.0, integ._stream),
                  "pp_fused_step")
            parity[0] ^= 1
        results[f"{name}/{variant}"] = time_launches(launch, stream, warmup,
                                                     reps)
    stream.synchronize()
    del keep
    return results


def _apply(integ, choice):
    layout, variant = choice.split("/")
    if layout == "untiled" and integ.tiling is not None:
        integ._drop_tiling()
    integ._fargs.variant = int(variant)


def tune_mixed(integ, warmup=3, reps=10):
    """Pick the layout and tile shape of a mixed-precision integrator.

    Times every tile shape of the untiled kernel and, when the integrator
    was set up tiled, of the tiled kernel, and keeps the fastest: an
    integrator whose untiled kernel wins drops its tiling.

    :returns: dict ``"layout/variant"`` -> milliseconds per step.
    """
    import torch
    fa = integ._fargs
    tiled = integ.tiling is not None
    key = ("mixed", fa.nnodes, fa.max_neigh, fa.integrator,
           bool(fa.stiffness_corrections), bool(fa.bond_types),
           bool(fa.node_instance), fa.flags, tiled)
    if key in _cache:
        _apply(integ, _cache[key][0])
        return _cache[key][1]
    with integ.context.on_stream():
        results = {}
        if tiled:
            results.update(_time_layout(integ, True, warmup, reps))
        results.update(_time_layout(integ, False, warmup, reps))
        best = min(results, key=results.get)
        _apply(integ, best)
    _cache[key] = (best, results)
    torch.cuda.empty_cache()
    return results
