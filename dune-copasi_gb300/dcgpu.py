"""ctypes binding of libdcgpu (include/dcgpu.h), mirroring the reference's model / stepper API.

The reference drives a simulation as (src/dune_copasi.cc:381-437):
    model = DiffusionReaction::make_model<Model>(config, functor_factory)
    state = model->make_state(grid, config); model->interpolate(state, model->make_initial(...))
    step_operator = model->make_step_operator(state, config)
    stepper.evolve(step_operator, state, state, dt, end_time, callback)
``Model`` below bundles make_model + make_state + interpolate + make_step_operator (the
state lives on the GPU), ``Model.step`` is SimpleAdaptiveStepper::do_step and
``Model.evolve`` is TimeStepper::evolve.  Errors raise ``DcError`` with the library's
message, as the reference raises format_exception(...).

There is no CPU fallback: constructing a model without the compiled library or without
a CUDA device raises.
"""

import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libdcgpu.so")

DC_OK = 0
STATUS_NAMES = {0: "DC_OK", 1: "DC_ERR_DIVERGED", 2: "DC_ERR_DT_MIN", 3: "DC_ERR_TIMEOUT",
                4: "DC_ERR_CONFIG", 5: "DC_ERR_CUDA", 6: "DC_ERR_ARGUMENT", 7: "DC_ERR_INTERNAL"}

EXPORTED = [
    "dc_model_create", "dc_model_destroy", "dc_model_info_get", "dc_species_name",
    "dc_species_size", "dc_species_vertices", "dc_state_set_initial", "dc_state_get",
    "dc_state_set", "dc_state_get_species", "dc_state_time", "dc_step", "dc_evolve",
    "dc_assemble", "dc_pattern", "dc_dof_map", "dc_stats", "dc_set_mixed_precision",
    "dc_expr_eval", "dc_stream_handle", "dc_launch_count", "dc_profile_enable", "dc_profile_get",
    "dc_assemble_residual_noalloc", "dc_server_create", "dc_server_submit", "dc_server_poll",
    "dc_server_take_state", "dc_server_estimate", "dc_server_destroy", "dc_last_error",
    "dc_spmv_format", "dc_vertex_coords", "dc_constraints", "dc_reduce", "dc_write_vtk", "dc_config_get",
    "dc_selftest_barrier_timeout", "dc_step_stage_newton", "dc_selftest_fma_peaks", "dc_jit_selftest",
    "dc_model_jit_status", "dc_precond_info", "dc_jacobian_apply", "dc_selftest_color", "dc_selftest_aggregate", "dc_selftest_precond",
    "dc_server_create_ex", "dc_server_batch_stats", "dc_server_batch_tuning",
]

SERVER_BATCH_KRYLOV = 1


class BatchStats(ctypes.Structure):
    _fields_ = [("solves", ctypes.c_int64), ("replays", ctypes.c_int64), ("slot_replays", ctypes.c_int64),
                ("iterations", ctypes.c_int64), ("max_active", ctypes.c_int32), ("reserved", ctypes.c_int32),
                ("replay_s", ctypes.c_double), ("wait_s", ctypes.c_double)]


class ReduceValue(ctypes.Structure):
    _fields_ = [("key", ctypes.c_char * 64), ("value", ctypes.c_double), ("error", ctypes.c_int32),
                ("warn", ctypes.c_int32)]


class DcError(RuntimeError):
    def __init__(self, status, message):
        super().__init__("%s: %s" % (STATUS_NAMES.get(status, status), message))
        self.status = status


class ModelInfo(ctypes.Structure):
    _fields_ = [("dim", ctypes.c_int32), ("n_species", ctypes.c_int32),
                ("n_compartments", ctypes.c_int32), ("block_size", ctypes.c_int32),
                ("n_vertices", ctypes.c_int64), ("n_elements", ctypes.c_int64),
                ("n_dof", ctypes.c_int64), ("n_block_rows", ctypes.c_int64),
                ("n_blocks", ctypes.c_int64)]


class StepInfo(ctypes.Structure):
    _fields_ = [("time", ctypes.c_double), ("dt_used", ctypes.c_double),
                ("newton_iterations", ctypes.c_int32), ("linear_iterations", ctypes.c_int32),
                ("failed_attempts", ctypes.c_int32), ("status", ctypes.c_int32),
                ("device_ms", ctypes.c_double)]


class Result(ctypes.Structure):
    _fields_ = [("request_id", ctypes.c_int64), ("status", ctypes.c_int32), ("reserved", ctypes.c_int32),
                ("queue_s", ctypes.c_double), ("run_s", ctypes.c_double), ("latency_s", ctypes.c_double),
                ("n_dof", ctypes.c_int64), ("newton_iterations", ctypes.c_int64),
                ("linear_iterations", ctypes.c_int64), ("steps", ctypes.c_int64),
                ("bytes_estimate", ctypes.c_int64), ("bytes_measured", ctypes.c_int64), ("setup_s", ctypes.c_double)]


CALLBACK = ctypes.CFUNCTYPE(None, ctypes.c_void_p, ctypes.c_double, ctypes.c_void_p)

_lib = None


def load_library(path=LIB_PATH):
    """Load libdcgpu.so and declare every exported entry point (raises if missing)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise ImportError("libdcgpu.so not built (run __graft_entry__.build()): %s" % path)
    lib = ctypes.CDLL(path)
    for name in EXPORTED:
        if not hasattr(lib, name):
            raise ImportError("libdcgpu.so lacks symbol %s" % name)
    P = ctypes.POINTER
    vp = ctypes.c_void_p
    d = ctypes.c_double
    i32 = ctypes.c_int32
    sz = ctypes.c_size_t
    pd = P(ctypes.c_double)
    lib.dc_model_create.argtypes = [ctypes.c_char_p, ctypes.c_char_p, P(vp)]
    lib.dc_model_destroy.argtypes = [vp]
    lib.dc_step_stage_newton.argtypes = [vp, P(ctypes.c_int32), sz, P(sz)]
    lib.dc_selftest_fma_peaks.argtypes = [pd, pd]
    lib.dc_jit_selftest.argtypes = [ctypes.c_char_p, sz]
    pi32 = ctypes.POINTER(ctypes.c_int32)
    lib.dc_selftest_color.argtypes = [ctypes.c_int64, pi32, pi32, pi32, pi32]
    lib.dc_selftest_aggregate.argtypes = [ctypes.c_int64, pi32, pi32, pi32, ctypes.c_int32, pi32,
                                          ctypes.POINTER(ctypes.c_int64)]
    lib.dc_selftest_precond.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int64, ctypes.c_int32, pi32, pi32,
                                        pd, pi32, pd, pd, ctypes.c_int32, pd]
    lib.dc_model_jit_status.argtypes = [vp, ctypes.c_char_p, sz]
    lib.dc_precond_info.argtypes = [vp, ctypes.c_char_p, sz]
    lib.dc_jacobian_apply.argtypes = [vp, pd, ctypes.c_double, ctypes.c_double, ctypes.c_double, pd, pd]
    lib.dc_model_info_get.argtypes = [vp, P(ModelInfo)]
    lib.dc_species_name.argtypes = [vp, i32, ctypes.c_char_p, sz]
    lib.dc_species_size.argtypes = [vp, i32, P(ctypes.c_int64)]
    lib.dc_species_vertices.argtypes = [vp, i32, P(ctypes.c_int64), sz]
    lib.dc_state_set_initial.argtypes = [vp]
    lib.dc_state_get.argtypes = [vp, pd, sz]
    lib.dc_state_set.argtypes = [vp, pd, sz, d]
    lib.dc_state_get_species.argtypes = [vp, i32, pd, sz]
    lib.dc_state_time.argtypes = [vp, pd]
    lib.dc_step.argtypes = [vp, pd, P(StepInfo)]
    lib.dc_evolve.argtypes = [vp, d, pd, CALLBACK, vp]
    lib.dc_assemble.argtypes = [vp, pd, d, d, d, pd, pd, sz]
    lib.dc_pattern.argtypes = [vp, P(ctypes.c_int32), sz, P(ctypes.c_int32), sz]
    lib.dc_dof_map.argtypes = [vp, P(ctypes.c_int64), sz]
    lib.dc_stats.argtypes = [vp, P(ctypes.c_int64), P(ctypes.c_int64), P(ctypes.c_int64), P(ctypes.c_int64)]
    lib.dc_set_mixed_precision.argtypes = [vp, ctypes.c_int]
    lib.dc_expr_eval.argtypes = [ctypes.c_char_p, ctypes.c_char_p, P(ctypes.c_char_p), pd, i32, pd]
    lib.dc_assemble_residual_noalloc.argtypes = [vp, pd, d, d, d, pd]
    lib.dc_server_create.argtypes = [ctypes.c_int64, i32, P(vp)]
    lib.dc_server_create_ex.argtypes = [ctypes.c_int64, i32, i32, P(vp)]
    lib.dc_server_batch_stats.argtypes = [vp, P(BatchStats)]
    lib.dc_server_batch_tuning.argtypes = [vp, ctypes.c_char_p, sz]
    lib.dc_server_submit.argtypes = [vp, ctypes.c_char_p, ctypes.c_char_p, pd, sz, P(ctypes.c_int64)]
    lib.dc_server_poll.argtypes = [vp, i32, P(Result), i32, P(i32)]
    lib.dc_server_take_state.argtypes = [vp, ctypes.c_int64, pd, sz]
    lib.dc_server_estimate.argtypes = [ctypes.c_char_p, ctypes.c_char_p, P(ctypes.c_int64)]
    lib.dc_server_destroy.argtypes = [vp]
    lib.dc_stream_handle.argtypes = [vp, P(vp)]
    lib.dc_launch_count.argtypes = []
    lib.dc_profile_enable.argtypes = [vp, ctypes.c_int]
    lib.dc_profile_get.argtypes = [vp, pd, P(ctypes.c_int64), i32]
    lib.dc_spmv_format.argtypes = [vp, P(i32), pd, pd]
    lib.dc_vertex_coords.argtypes = [vp, pd, sz]
    lib.dc_constraints.argtypes = [vp, P(ctypes.c_int64), pd, sz, P(sz)]
    lib.dc_reduce.argtypes = [vp, ctypes.c_char_p, P(ReduceValue), sz, P(sz)]
    lib.dc_write_vtk.argtypes = [vp, ctypes.c_char_p, ctypes.c_int]
    lib.dc_config_get.argtypes = [vp, ctypes.c_char_p, ctypes.c_char_p, sz]
    lib.dc_selftest_barrier_timeout.argtypes = [pd, pd]
    lib.dc_last_error.argtypes = []
    lib.dc_last_error.restype = ctypes.c_char_p
    for name in EXPORTED:
        if name not in ("dc_last_error", "dc_launch_count"):
            getattr(lib, name).restype = ctypes.c_int
    lib.dc_launch_count.restype = ctypes.c_int64
    _lib = lib
    return lib


def _check(status):
    if status != DC_OK:
        msg = _lib.dc_last_error().decode(errors="replace")
        raise DcError(status, msg)


def expr_eval(expression, variables=None, context_ini=None):
    """Evaluate one expression on the host with the engine's compiler (no GPU needed)."""
    lib = load_library()
    variables = variables or {}
    names = list(variables)
    arr_n = (ctypes.c_char_p * max(len(names), 1))(*[n.encode() for n in names])
    vals = np.array([float(variables[n]) for n in names] or [0.0])
    out = ctypes.c_double()
    _check(lib.dc_expr_eval(expression.encode(), context_ini.encode() if context_ini else None, arr_n,
                            vals.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), len(names),
                            ctypes.byref(out)))
    return out.value


def _ptr(a, ctype=ctypes.c_double):
    return a.ctypes.data_as(ctypes.POINTER(ctype))


class Model:
    """A DuneCopasi diffusion-reaction model resident on the GPU.

    ``ini`` is the configuration text; ``overrides`` maps keys to values (the CLI's
    ``--key=value``).
    """

    def __init__(self, ini, overrides=None):
        lib = load_library()
        self._lib = lib
        ov = None
        if overrides:
            ov = "\n".join("%s=%s" % (k, v) for k, v in overrides.items()).encode()
        h = ctypes.c_void_p()
        _check(lib.dc_model_create(ini.encode(), ov, ctypes.byref(h)))
        self._h = h
        info = ModelInfo()
        _check(lib.dc_model_info_get(h, ctypes.byref(info)))
        self.info = {f: getattr(info, f) for f, _ in ModelInfo._fields_}
        self.species = []
        buf = ctypes.create_string_buffer(256)
        for s in range(info.n_species):
            _check(lib.dc_species_name(h, s, buf, 256))
            self.species.append(buf.value.decode())

    # -- lifetime
    def close(self):
        if getattr(self, "_h", None):
            _check(self._lib.dc_model_destroy(self._h))
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # -- state
    @property
    def ndof(self):
        return self.info["n_dof"]

    def state(self, out=None):
        """The state in the reference DOF layout; `out` (float64, ndof, contiguous) is filled
        in place when given (e.g. a pinned host array)."""
        if out is None:
            out = np.empty(self.ndof)
        elif out.dtype != np.float64 or out.size != self.ndof or not out.flags["C_CONTIGUOUS"]:
            raise ValueError("out must be a contiguous float64 array of ndof values")
        _check(self._lib.dc_state_get(self._h, _ptr(out), out.size))
        return out

    def set_state(self, x, time):
        x = np.ascontiguousarray(x, dtype=np.float64)
        _check(self._lib.dc_state_set(self._h, _ptr(x), x.size, float(time)))

    def set_initial(self):
        _check(self._lib.dc_state_set_initial(self._h))

    def time(self):
        t = ctypes.c_double()
        _check(self._lib.dc_state_time(self._h, ctypes.byref(t)))
        return t.value

    def species_index(self, name):
        return self.species.index(name)

    def species_vertices(self, name):
        s = self.species_index(name)
        n = ctypes.c_int64()
        _check(self._lib.dc_species_size(self._h, s, ctypes.byref(n)))
        out = np.empty(n.value, np.int64)
        _check(self._lib.dc_species_vertices(self._h, s, _ptr(out, ctypes.c_int64), out.size))
        return out

    def vertex_coords(self):
        """(n_vertices, dim) vertex coordinates of the grid."""
        out = np.empty((self.info["n_vertices"], self.info["dim"]))
        _check(self._lib.dc_vertex_coords(self._h, _ptr(out), out.size))
        return out

    def config_get(self, key):
        """Value of a configuration key (after overrides), or None when absent."""
        buf = ctypes.create_string_buffer(4096)
        st = self._lib.dc_config_get(self._h, key.encode(), buf, 4096)
        return buf.value.decode() if st == DC_OK else None

    def write_vtk(self, path, append=True):
        """VTK output of the current state: per compartment <path>/<stem>-<compartment>-NNNNN.vtu
        and the time series <path>/<stem>-<compartment>.pvd."""
        _check(self._lib.dc_write_vtk(self._h, str(path).encode(), 1 if append else 0))

    def reduce(self, reduce_ini=None):
        """Transform/reduce operators on the current state: ({key: value}, [error keys],
        [warning keys]); reduce_ini None uses the model's [model.reduce] section."""
        text = reduce_ini.encode() if reduce_ini is not None else None
        n = ctypes.c_size_t(0)
        _check(self._lib.dc_reduce(self._h, text, None, 0, ctypes.byref(n)))
        arr = (ReduceValue * max(n.value, 1))()
        _check(self._lib.dc_reduce(self._h, text, arr, n.value, ctypes.byref(n)))
        vals, errs, warns = {}, [], []
        for k in range(n.value):
            key = arr[k].key.decode()
            vals[key] = arr[k].value
            if arr[k].error:
                errs.append(key)
            elif arr[k].warn:
                warns.append(key)
        return vals, errs, warns

    def constraints(self):
        """(reference DOF indices, values) of the Dirichlet constraints, sorted by DOF."""
        n = ctypes.c_size_t(0)
        _check(self._lib.dc_constraints(self._h, None, None, 0, ctypes.byref(n)))
        dofs = np.empty(n.value, np.int64)
        vals = np.empty(n.value)
        if n.value:
            _check(self._lib.dc_constraints(self._h, _ptr(dofs, ctypes.c_int64), _ptr(vals), n.value,
                                            ctypes.byref(n)))
        order = np.argsort(dofs, kind="stable")
        return dofs[order], vals[order]

    def _layout(self):
        """[(species names of one compartment, vertex ids, first DOF)] in DOF order
        (compartment-major, vertex-major, species interleaved)."""
        out, off, i = [], 0, 0
        names = self.species
        while i < len(names):
            verts = self.species_vertices(names[i])
            group = [names[i]]
            while i + len(group) < len(names) and \
                    np.array_equal(self.species_vertices(names[i + len(group)]), verts):
                group.append(names[i + len(group)])
            out.append((group, verts, off))
            off += len(group) * len(verts)
            i += len(group)
        return out

    def species_dofs(self, name):
        """Indices of a species' DOFs in the reference-order state vector."""
        for group, verts, off in self._layout():
            if name in group:
                return off + group.index(name) + len(group) * np.arange(len(verts))
        raise KeyError(name)

    def seeded_state(self, init):
        """State vector (reference DOF order) with init(species name, vertex coords) per
        species; species for which init returns None keep their initial.expression values."""
        x = self.state()
        if init is None:
            return x
        coords = self.vertex_coords()
        off = 0
        names = self.species
        i = 0
        while i < len(names):
            verts = self.species_vertices(names[i])
            group = [names[i]]
            while i + len(group) < len(names) and \
                    np.array_equal(self.species_vertices(names[i + len(group)]), verts):
                group.append(names[i + len(group)])
            ns = len(group)
            for k, name in enumerate(group):
                v = init(name, coords[verts])
                if v is not None:
                    x[off + k: off + ns * len(verts): ns] = v
            off += ns * len(verts)
            i += ns
        return x

    def species_values(self, name):
        s = self.species_index(name)
        n = ctypes.c_int64()
        _check(self._lib.dc_species_size(self._h, s, ctypes.byref(n)))
        out = np.empty(n.value)
        _check(self._lib.dc_state_get_species(self._h, s, _ptr(out), out.size))
        return out

    # -- stepping (SimpleAdaptiveStepper / TimeStepper)
    def step(self, dt):
        """One adaptive step; returns a dict with the step statistics and the next dt."""
        d = ctypes.c_double(dt)
        info = StepInfo()
        st = self._lib.dc_step(self._h, ctypes.byref(d), ctypes.byref(info))
        _check(st)
        out = {f: getattr(info, f) for f, _ in StepInfo._fields_}
        out["dt_next"] = d.value
        out["newton_per_stage"] = self.stage_newton()
        return out

    def jit_status(self):
        """"compiled", "off" or "interpreter (<reason>)": the model's volume kernels."""
        buf = ctypes.create_string_buffer(4096)
        _check(self._lib.dc_model_jit_status(self._h, buf, len(buf)))
        return buf.value.decode()

    def precond_info(self):
        """The preconditioner of the linear solves (dict): type and structure (colours, or
        rows / blocks / kernel kind of every multigrid level)."""
        import json
        buf = ctypes.create_string_buffer(16384)
        _check(self._lib.dc_precond_info(self._h, buf, len(buf)))
        return json.loads(buf.value.decode())

    def stage_newton(self):
        """Newton iterations of every stage solve of the last step (dc_step_stage_newton)."""
        n = ctypes.c_size_t()
        _check(self._lib.dc_step_stage_newton(self._h, None, 0, ctypes.byref(n)))
        buf = (ctypes.c_int32 * max(n.value, 1))()
        _check(self._lib.dc_step_stage_newton(self._h, buf, n.value, ctypes.byref(n)))
        return [int(buf[i]) for i in range(n.value)]

    def evolve(self, t_end, dt, callback=None):
        d = ctypes.c_double(dt)

        def _cb(_m, t, _u):
            if callback is not None:
                callback(t)

        cb = CALLBACK(_cb)
        _check(self._lib.dc_evolve(self._h, float(t_end), ctypes.byref(d), cb, None))
        return d.value

    # -- operator access
    def _state_arg(self, x):
        """x as a C-contiguous float64 vector of n_dof values (the C ABI copies n_dof values
        from it and takes no length)."""
        x = np.ascontiguousarray(x, dtype=np.float64)
        if x.ndim != 1 or x.size != self.ndof:
            raise ValueError("state vector must hold %d values, got shape %s" % (self.ndof, x.shape))
        return x

    def _out_arg(self, out):
        """A caller's output vector: it must be a writable C-contiguous float64 array of n_dof
        values, since the C ABI writes n_dof values into it."""
        if out is None:
            return np.empty(self.ndof)
        if (not isinstance(out, np.ndarray) or out.dtype != np.float64 or not out.flags.c_contiguous
                or not out.flags.writeable or out.size != self.ndof):
            raise ValueError("out must be a writable C-contiguous float64 array of %d values" % self.ndof)
        return out

    def assemble(self, x, t, cm, ca, residual=True, jacobian=True):
        x = self._state_arg(x)
        r = np.empty(self.ndof) if residual else None
        bs = self.info["block_size"]
        nj = self.info["n_blocks"] * bs * bs
        J = np.empty(nj) if jacobian else None
        _check(self._lib.dc_assemble(self._h, _ptr(x), float(t), float(cm), float(ca),
                                     _ptr(r) if r is not None else None,
                                     _ptr(J) if J is not None else None, nj if J is not None else 0))
        return r, J

    def jacobian_apply(self, x, t, cm, ca, v):
        """Matrix-free product (cm dM/dx + ca dA/dx)(x, t) v, reference order (dc_jacobian_apply)."""
        x = self._state_arg(x)
        v = self._state_arg(v)
        y = np.zeros(self.ndof)
        P = ctypes.POINTER(ctypes.c_double)
        _check(self._lib.dc_jacobian_apply(self._h, x.ctypes.data_as(P), float(t), float(cm), float(ca),
                                           v.ctypes.data_as(P), y.ctypes.data_as(P)))
        return y

    def residual_noalloc(self, x, t, cm, ca, out=None):
        """Residual through the allocation-free entry point (staging in the library's fixed
        device array; see include/dcgpu.h).  Returns the residual, or raises DcError."""
        x = self._state_arg(x)
        r = self._out_arg(out)
        st = self._lib.dc_assemble_residual_noalloc(self._h, _ptr(x), float(t), float(cm), float(ca), _ptr(r))
        if st != DC_OK:
            raise DcError(st, "dc_assemble_residual_noalloc failed")
        return r

    def pattern(self):
        nr = self.info["n_block_rows"]
        rowptr = np.empty(nr + 1, np.int32)
        colidx = np.empty(self.info["n_blocks"], np.int32)
        _check(self._lib.dc_pattern(self._h, _ptr(rowptr, ctypes.c_int32), rowptr.size,
                                    _ptr(colidx, ctypes.c_int32), colidx.size))
        return rowptr, colidx

    def dof_map(self):
        out = np.empty(self.ndof, np.int64)
        _check(self._lib.dc_dof_map(self._h, _ptr(out, ctypes.c_int64), out.size))
        return out

    def jacobian_csr(self, J):
        """Expand BSR values into a scipy CSR matrix in the reference DOF order."""
        import scipy.sparse as sp
        rowptr, colidx = self.pattern()
        bs = self.info["block_size"]
        nr = self.info["n_block_rows"]
        blocks = J.reshape(-1, bs, bs)
        brow = np.repeat(np.arange(nr), np.diff(rowptr))
        rows = (brow[:, None, None] * bs + np.arange(bs)[None, :, None]).repeat(bs, axis=2)
        cols = (colidx[:, None, None] * bs + np.arange(bs)[None, None, :]).repeat(bs, axis=1)
        A = sp.csr_matrix((blocks.ravel(), (rows.ravel(), cols.ravel())), shape=(nr * bs, nr * bs))
        m = self.dof_map()
        return A[m][:, m]

    def stats(self):
        v = [ctypes.c_int64() for _ in range(4)]
        _check(self._lib.dc_stats(self._h, *[ctypes.byref(x) for x in v]))
        return dict(zip(("newton_iterations", "linear_iterations", "assemblies", "failed_steps"),
                        [x.value for x in v]))

    def set_mixed_precision(self, enabled):
        _check(self._lib.dc_set_mixed_precision(self._h, 1 if enabled else 0))

    # -- instrumentation
    def stream_handle(self):
        s = ctypes.c_void_p()
        _check(self._lib.dc_stream_handle(self._h, ctypes.byref(s)))
        return s.value or 0

    def profile(self, enabled=True):
        _check(self._lib.dc_profile_enable(self._h, 1 if enabled else 0))

    def kernel_times(self):
        """{category: (total ms, launches)} for assembly (all passes), spmv, precond,
        krylov_iteration (single-launch BiCGSTAB solves; its count is the Krylov iterations
        they ran) and the assembly passes by kind: assembly_residual, assembly_jacobian,
        assembly_combined."""
        names = ("assembly_residual", "spmv", "precond", "krylov_iteration", "assembly_jacobian",
                 "assembly_combined")
        ms = np.zeros(len(names))
        calls = np.zeros(len(names), np.int64)
        _check(self._lib.dc_profile_get(self._h, _ptr(ms), _ptr(calls, ctypes.c_int64), len(names)))
        out = {k: (float(ms[i]), int(calls[i])) for i, k in enumerate(names)}
        parts = ("assembly_residual", "assembly_jacobian", "assembly_combined")
        out["assembly"] = (sum(out[k][0] for k in parts), sum(out[k][1] for k in parts))
        return out

    def spmv_format(self):
        """Layout of the fp32 Krylov operator and the tuner's SpMV times:
        {"format": "auto"|"bsr"|"sell", "bsr_us": t, "sell_us": t}."""
        f = ctypes.c_int32(0)
        a = ctypes.c_double(0.0)
        b = ctypes.c_double(0.0)
        _check(self._lib.dc_spmv_format(self._h, ctypes.byref(f), ctypes.byref(a), ctypes.byref(b)))
        return {"format": {-1: "auto", 0: "bsr", 1: "sell"}[f.value], "bsr_us": a.value, "sell_us": b.value}


def launch_count():
    return int(load_library().dc_launch_count())


def jit_selftest():
    """(ok, message) of the run-time compilation self-test (NVRTC, no GPU needed)."""
    lib = load_library()
    buf = ctypes.create_string_buffer(8192)
    st = lib.dc_jit_selftest(buf, len(buf))
    return st == DC_OK, buf.value.decode()


def fma_peaks():
    """(FP64, FP32) fused multiply-add throughput of the current device in TFLOP/s."""
    lib = load_library()
    d = ctypes.c_double(0.0)
    f = ctypes.c_double(0.0)
    _check(lib.dc_selftest_fma_peaks(ctypes.byref(d), ctypes.byref(f)))
    return d.value, f.value


def _i32(a):
    a = np.ascontiguousarray(a, dtype=np.int32)
    return a, a.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))


def _f64(a):
    a = np.ascontiguousarray(a, dtype=np.float64)
    return a, a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _check_csr(rowptr, colidx, group=None):
    """The C entry points read rowptr[n] column indices and n group entries and take no
    lengths: check them here."""
    rowptr = np.asarray(rowptr)
    if rowptr.ndim != 1 or rowptr.size < 2:
        raise ValueError("rowptr must hold n + 1 >= 2 offsets")
    if len(colidx) != int(rowptr[-1]):
        raise ValueError("colidx must hold rowptr[-1] = %d entries, got %d" % (int(rowptr[-1]), len(colidx)))
    if group is not None and len(group) != rowptr.size - 1:
        raise ValueError("group must hold one entry per row")


def color_graph(rowptr, colidx):
    """(colour per row, number of colours) of the multicolour preconditioners' colouring."""
    _check_csr(rowptr, colidx)
    lib = load_library()
    n = len(rowptr) - 1
    rp, prp = _i32(rowptr)
    ci, pci = _i32(colidx)
    out = np.zeros(n, np.int32)
    nc = ctypes.c_int32(0)
    _check(lib.dc_selftest_color(n, prp, pci, out.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), ctypes.byref(nc)))
    return out, nc.value


def aggregate_graph(rowptr, colidx, group=None, distance=2):
    """(aggregate per row, number of aggregates) of one multigrid coarsening."""
    _check_csr(rowptr, colidx, group)
    lib = load_library()
    n = len(rowptr) - 1
    rp, prp = _i32(rowptr)
    ci, pci = _i32(colidx)
    if group is not None:
        g, pg = _i32(group)
    else:
        pg = None
    out = np.zeros(n, np.int32)
    na = ctypes.c_int64(0)
    _check(lib.dc_selftest_aggregate(n, prp, pci, pg, int(distance), out.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                                     ctypes.byref(na)))
    return out, int(na.value)


def precond_apply(kind, rowptr, colidx, vals, r, bs, params="", group=None, fp32=False):
    """z = M^-1 r for preconditioner `kind` built on the BSR matrix (vals: nnzb x bs x bs);
    returns (z, info) with info as dc_selftest_precond describes."""
    _check_csr(rowptr, colidx, group)
    n = len(rowptr) - 1
    if np.asarray(vals).size != len(colidx) * bs * bs or np.asarray(r).size != n * bs:
        raise ValueError("vals must hold nnzb * bs * bs values and r n * bs values")
    lib = load_library()
    rp, prp = _i32(rowptr)
    ci, pci = _i32(colidx)
    v, pv = _f64(np.asarray(vals).reshape(-1))
    rr, pr = _f64(r)
    if group is not None:
        g, pg = _i32(group)
    else:
        pg = None
    z = np.zeros(n * bs)
    info = np.zeros(8)
    _check(lib.dc_selftest_precond(kind.encode(), params.encode(), n, int(bs), prp, pci, pv, pg, pr,
                                   z.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), 1 if fp32 else 0,
                                   info.ctypes.data_as(ctypes.POINTER(ctypes.c_double))))
    return z, info


def selftest_barrier_timeout():
    """Runs one grid-wide barrier that cannot complete (4 cooperative blocks, 50 ms limit)
    and returns (blocks whose wait gave up, kernel milliseconds)."""
    lib = load_library()
    gave = ctypes.c_double(0.0)
    ms = ctypes.c_double(0.0)
    _check(lib.dc_selftest_barrier_timeout(ctypes.byref(gave), ctypes.byref(ms)))
    return gave.value, ms.value


def estimate_bytes(ini, overrides=None):
    """Device footprint the server's admission control assumes for a request (host only)."""
    lib = load_library()
    ov = "\n".join("%s=%s" % (k, v) for k, v in overrides.items()).encode() if overrides else None
    b = ctypes.c_int64()
    _check(lib.dc_server_estimate(ini.encode(), ov, ctypes.byref(b)))
    return b.value


class Server:
    """Request server: admits simulations by device-memory budget and runs them concurrently.

    ``submit`` returns a request id; ``poll`` returns completed results as dicts;
    ``take_state`` returns the final state of a completed request.  With ``batch_krylov``
    the running simulations' block-Jacobi BiCGSTAB solves are packed into one continuously
    batched solve (``batch_stats`` reports its counters).
    """

    def __init__(self, budget_bytes, max_active=4, batch_krylov=False):
        self._lib = load_library()
        h = ctypes.c_void_p()
        flags = SERVER_BATCH_KRYLOV if batch_krylov else 0
        _check(self._lib.dc_server_create_ex(int(budget_bytes), int(max_active), flags, ctypes.byref(h)))
        self._h = h
        self._ndof = {}

    def submit(self, ini, overrides=None, init=None):
        ov = "\n".join("%s=%s" % (k, v) for k, v in overrides.items()).encode() if overrides else None
        rid = ctypes.c_int64()
        if init is not None:
            init = np.ascontiguousarray(init, dtype=np.float64)
            _check(self._lib.dc_server_submit(self._h, ini.encode(), ov, _ptr(init), init.size, ctypes.byref(rid)))
        else:
            _check(self._lib.dc_server_submit(self._h, ini.encode(), ov, None, 0, ctypes.byref(rid)))
        return rid.value

    def poll(self, wait=True, max_results=64):
        arr = (Result * max_results)()
        n = ctypes.c_int32()
        _check(self._lib.dc_server_poll(self._h, 1 if wait else 0, arr, max_results, ctypes.byref(n)))
        out = []
        for i in range(n.value):
            r = {f: getattr(arr[i], f) for f, _ in Result._fields_}
            self._ndof[r["request_id"]] = r["n_dof"]
            out.append(r)
        return out

    def take_state(self, request_id):
        n = self._ndof.get(request_id)
        if n is None:
            raise KeyError(request_id)
        out = np.empty(n)
        _check(self._lib.dc_server_take_state(self._h, int(request_id), _ptr(out), out.size))
        return out

    def batch_stats(self):
        st = BatchStats()
        _check(self._lib.dc_server_batch_stats(self._h, ctypes.byref(st)))
        return {f: getattr(st, f) for f, _ in BatchStats._fields_ if f != "reserved"}

    def batch_tuning(self):
        """Replay grid the batch's autotuner chose per batch-size bucket and precision."""
        import json
        buf = ctypes.create_string_buffer(4096)
        _check(self._lib.dc_server_batch_tuning(self._h, buf, len(buf)))
        return json.loads(buf.value.decode())

    def close(self):
        if getattr(self, "_h", None):
            _check(self._lib.dc_server_destroy(self._h))
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
