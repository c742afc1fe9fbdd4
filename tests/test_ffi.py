"""The XLA FFI handlers (aj_ffi_prepare, aj_ffi_step) against hand-built call
frames in the typed-FFI C layout (xla/ffi/api/c_api.h, API version 0): a
fake API table whose XLA_FFI_Error_Create records the message and code and
whose XLA_FFI_Stream_Get hands out a stream.

CPU: every rejection happens on the host before anything is enqueued -
missing or malformed attributes, buffer types and sizes, the reference's
multigrid shape rule (multigrid_solver.py:96-106) through aj_check_params,
short workspaces - and stages other than execute do nothing.
GPU: aj_ffi_prepare + aj_ffi_step on device buffers give bit for bit the
fields of aj_step through the Python API."""
import ctypes
from ctypes import POINTER, c_char_p, c_int32, c_int64, c_size_t, c_void_p

import numpy as np
import pytest

F32, U8 = 11, 6
BUFFER, ARRAY = 1, 1
EXECUTE, INSTANTIATE = 3, 0


class Buffer(ctypes.Structure):
    _fields_ = [("struct_size", c_size_t), ("ext", c_void_p), ("dtype", c_int32),
                ("data", c_void_p), ("rank", c_int64), ("dims", POINTER(c_int64))]


class Args(ctypes.Structure):
    _fields_ = [("struct_size", c_size_t), ("ext", c_void_p), ("size", c_int64),
                ("types", POINTER(c_int32)), ("args", POINTER(c_void_p))]


class ByteSpan(ctypes.Structure):
    _fields_ = [("ptr", c_char_p), ("len", c_size_t)]


class Array(ctypes.Structure):
    _fields_ = [("dtype", c_int32), ("size", c_size_t), ("data", c_void_p)]


class Attrs(ctypes.Structure):
    _fields_ = [("struct_size", c_size_t), ("ext", c_void_p), ("size", c_int64),
                ("types", POINTER(c_int32)), ("names", POINTER(POINTER(ByteSpan))),
                ("attrs", POINTER(c_void_p))]


class ErrorCreateArgs(ctypes.Structure):
    _fields_ = [("struct_size", c_size_t), ("ext", c_void_p), ("message", c_char_p),
                ("errc", c_int32)]


class StreamGetArgs(ctypes.Structure):
    _fields_ = [("struct_size", c_size_t), ("ext", c_void_p), ("ctx", c_void_p),
                ("stream", c_void_p)]


class ApiVersion(ctypes.Structure):
    _fields_ = [("struct_size", c_size_t), ("ext", c_void_p), ("major", c_int32),
                ("minor", c_int32)]


ERR_FN = ctypes.CFUNCTYPE(c_void_p, POINTER(ErrorCreateArgs))
STREAM_FN = ctypes.CFUNCTYPE(c_void_p, POINTER(StreamGetArgs))


class Api(ctypes.Structure):
    _fields_ = [("struct_size", c_size_t), ("ext", c_void_p), ("version", ApiVersion),
                ("internal", c_void_p), ("error_create", ERR_FN), ("error_get_message", c_void_p),
                ("error_destroy", c_void_p), ("handler_register", c_void_p),
                ("stream_get", STREAM_FN)]


class CallFrame(ctypes.Structure):
    _fields_ = [("struct_size", c_size_t), ("ext", c_void_p), ("api", POINTER(Api)),
                ("ctx", c_void_p), ("stage", c_int32), ("args", Args), ("rets", Args),
                ("attrs", Attrs)]


class Frame:
    """A call frame plus everything it points to (kept alive here)."""

    def __init__(self, args, rets, params=None, stage=EXECUTE, stream=0, params_dtype=U8):
        self.errors = []
        self._keep = []

        def err(a):
            self.errors.append((a.contents.message.decode(), a.contents.errc))
            return 1                                  # any non-null pointer is an error

        def stream_get(a):
            a.contents.stream = stream
            return None
        self._err, self._stream = ERR_FN(err), STREAM_FN(stream_get)
        self.api = Api(ctypes.sizeof(Api), None, ApiVersion(ctypes.sizeof(ApiVersion), None, 0, 1),
                       None, self._err, None, None, None, self._stream)
        self.frame = CallFrame()
        self.frame.struct_size = ctypes.sizeof(CallFrame)
        self.frame.api = ctypes.pointer(self.api)
        self.frame.stage = stage
        self.frame.args = self._bufs(args)
        self.frame.rets = self._bufs(rets)
        if params is None:
            self.frame.attrs = Attrs(ctypes.sizeof(Attrs), None, 0, None, None, None)
        else:
            raw = np.ascontiguousarray(params)
            self._keep.append(raw)
            arr = Array(params_dtype, raw.size, raw.ctypes.data)
            name = ByteSpan(b"params", 6)
            self._keep += [arr, name]
            names = (POINTER(ByteSpan) * 1)(ctypes.pointer(name))
            types = (c_int32 * 1)(ARRAY)
            vals = (c_void_p * 1)(ctypes.addressof(arr))
            self._keep += [names, types, vals]
            self.frame.attrs = Attrs(ctypes.sizeof(Attrs), None, 1, types, names, vals)

    def _bufs(self, specs):
        bufs = []
        for dtype, ptr, dims in specs:
            d = (c_int64 * max(1, len(dims)))(*dims)
            b = Buffer(ctypes.sizeof(Buffer), None, dtype, ptr, len(dims), d)
            self._keep += [d, b]
            bufs.append(b)
        types = (c_int32 * max(1, len(bufs)))(*([BUFFER] * len(bufs)))
        ptrs = (c_void_p * max(1, len(bufs)))(*[ctypes.addressof(b) for b in bufs])
        self._keep += [types, ptrs]
        return Args(ctypes.sizeof(Args), None, len(bufs), types, ptrs)

    def call(self, fn):
        return fn(ctypes.addressof(self.frame))


@pytest.fixture(scope="module")
def L():
    from aerojax_gb300 import build, _lib
    build.build()
    return _lib.lib()


def _cfg(**kw):
    from aerojax_gb300.params import StepConfig
    base = dict(nx=512, ny=96, dx=1 / 64, dy=1 / 64, nu=1e-3, v_cycles=3, dt=1e-3,
                variant="gui")
    base.update(kw)
    return StepConfig(**base)


def _host(n, dtype=np.float32):
    a = np.zeros(n, dtype)
    return a, a.ctypes.data


def _step_frame(cfg, ws_bytes=1 << 20, u_dtype=F32, **kw):
    from aerojax_gb300 import jax_ffi
    nx, ny = cfg.nx, cfg.ny
    keep = []
    specs = []
    for n, dt in ((nx * ny, u_dtype), (nx * ny, F32), (nx * ny, F32), (0, F32)):
        a, p = _host(max(n, 1))
        keep.append(a)
        specs.append((dt, p, [n] if n else [0]))
    w, wp = _host(ws_bytes, np.uint8)
    keep.append(w)
    specs.append((U8, wp, [ws_bytes]))
    rets = []
    for _ in range(3):
        a, p = _host(nx * ny)
        keep.append(a)
        rets.append((F32, p, [nx, ny]))
    fr = Frame(specs, rets, params=kw.pop("params", jax_ffi.params_bytes(cfg)), **kw)
    fr._keep.append(keep)
    return fr


def test_handlers_exported(L):
    assert L.aj_ffi_step and L.aj_ffi_prepare


def test_non_execute_stage_does_nothing(L):
    fr = _step_frame(_cfg(), stage=INSTANTIATE)
    assert fr.call(L.aj_ffi_step) is None
    assert fr.errors == []


def test_missing_params_attribute(L):
    fr = _step_frame(_cfg(), params=None)
    fr.frame.attrs.size = 0
    assert fr.call(L.aj_ffi_step)
    msg, code = fr.errors[0]
    assert "params" in msg and code == 3


def test_params_of_the_wrong_size(L):
    fr = _step_frame(_cfg(), params=np.zeros(7, np.uint8))
    assert fr.call(L.aj_ffi_step)
    assert "params" in fr.errors[0][0]


def test_wrong_dtype(L):
    fr = _step_frame(_cfg(), u_dtype=U8)
    assert fr.call(L.aj_ffi_step)
    msg, code = fr.errors[0]
    assert "argument 0 must be float32" in msg and code == 3


def test_reference_shape_rule(L):
    """A grid the reference's multigrid rejects (ValueError,
    multigrid_solver.py:104-106) comes back as AJ_ERR_SHAPE from aj_check_params."""
    fr = _step_frame(_cfg(nx=100, ny=64))
    assert fr.call(L.aj_ffi_step)
    msg, code = fr.errors[0]
    assert "AJ_ERR_SHAPE" in msg and code == 3


def test_prepare_rejects_short_workspace(L):
    from aerojax_gb300 import jax_ffi
    cfg = _cfg()
    mask, mp = _host(cfg.nx * cfg.ny)
    sdf, sp = _host(1)
    ws, wp = _host(64, np.uint8)
    fr = Frame([(F32, mp, [cfg.nx, cfg.ny]), (F32, sp, [0])], [(U8, wp, [64])],
               params=jax_ffi.params_bytes(cfg))
    assert fr.call(L.aj_ffi_prepare)
    msg, code = fr.errors[0]
    assert "AJ_ERR_WORKSPACE" in msg and code == 8
    assert jax_ffi.workspace_bytes(cfg) > 64


@pytest.mark.gpu
def test_ffi_step_matches_python_api(cuda_lib):
    """aj_ffi_prepare + aj_ffi_step on device buffers (the stream handed out by
    the call frame's API) reproduce run_step bit for bit, three steps of the
    512x128 NACA workload with the converging solve."""
    from dataclasses import replace
    import torch
    import aerojax_gb300 as aj
    from aerojax_gb300 import configs, jax_ffi
    case = configs.naca_mac_2048x512(nx=512, ny=128, mg_mode="converge")
    cfg = replace(case["cfg"], warm_start=True)
    nx, ny = cfg.nx, cfg.ny
    stream = torch.cuda.current_stream().cuda_stream
    nbytes = jax_ffi.workspace_bytes(cfg)
    ws = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
    mask = case["mask"]
    empty = torch.empty(1, device="cuda")
    fr = Frame([(F32, mask.data_ptr(), [nx, ny]), (F32, empty.data_ptr(), [0])],
               [(U8, ws.data_ptr(), [nbytes])], params=jax_ffi.params_bytes(cfg), stream=stream)
    assert fr.call(cuda_lib.aj_ffi_prepare) is None, fr.errors
    plan = aj.Plan(cfg, torch.device("cuda"))
    plan.prepare(mask)
    u, v = case["u"].clone(), case["v"].clone()
    p = torch.zeros((nx, ny), device="cuda")
    fu, fv, fp = u.clone(), v.clone(), p.clone()
    for _ in range(3):
        u, v, p = aj.run_step(plan, u, v, mask, p_guess=p)
        outs = (torch.empty_like(fu), torch.empty_like(fv), torch.empty_like(fp))
        fr = Frame([(F32, fu.data_ptr(), list(fu.shape)), (F32, fv.data_ptr(), list(fv.shape)),
                    (F32, mask.data_ptr(), [nx, ny]), (F32, fp.data_ptr(), [nx, ny]),
                    (U8, ws.data_ptr(), [nbytes])],
                   [(F32, outs[0].data_ptr(), list(fu.shape)),
                    (F32, outs[1].data_ptr(), list(fv.shape)),
                    (F32, outs[2].data_ptr(), [nx, ny]), (U8, ws.data_ptr(), [nbytes])],
                   params=jax_ffi.params_bytes(cfg), stream=stream)
        assert fr.call(cuda_lib.aj_ffi_step) is None, fr.errors
        fu, fv, fp = outs
    torch.cuda.synchronize()
    assert torch.equal(fu, u) and torch.equal(fv, v) and torch.equal(fp, p)
