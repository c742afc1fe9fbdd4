// XLA FFI handlers: the C ABI as JAX custom calls, the binding of the
// reference's jit boundary (solver/simulation/step_handlers.py:304-315
// get_step_jit / jax.jit(self._step); solver/pure_functions/step.py:49
// step_pure's jit).  A JAX program registers them with
//   jax.ffi.register_ffi_target("aj_step", jax.ffi.pycapsule(lib.aj_ffi_step),
//                               platform="CUDA")
// and calls them through jax.ffi.ffi_call (aerojax_gb300/jax_ffi.py).
//
// The handlers read XLA's call frame through the typed-FFI C layout
// (xla/ffi/api/c_api.h, API version 0): every struct starts with its size and
// an extension pointer; buffers carry dtype, data pointer, rank and dims; the
// API table begins with struct_size, extension_start, api_version,
// internal_api, then the function pointers XLA_FFI_Error_Create,
// _Error_GetMessage, _Error_Destroy, _Handler_Register, _Stream_Get in that
// order.  Only the fields below are touched.  jaxlib's own header is not
// needed to build them (jaxlib is not required by this library); the layout
// is restated here, and each struct's size field is checked before use.
#include "aj_internal.cuh"
#include <string.h>
#include <stdio.h>

namespace aj {
namespace ffi {

struct ExtBase;
struct Api;
struct Ctx;
struct Error;

enum DataType : int32_t { DT_U8 = 6, DT_F32 = 11 };
enum ArgType : int32_t { ARG_BUFFER = 1 };
enum AttrType : int32_t { ATTR_ARRAY = 1, ATTR_DICT = 2, ATTR_SCALAR = 3, ATTR_STRING = 4 };
enum Stage : int32_t { STAGE_INSTANTIATE = 0, STAGE_PREPARE = 1, STAGE_INITIALIZE = 2,
                       STAGE_EXECUTE = 3 };
enum ErrorCode : int32_t { ERR_INVALID_ARGUMENT = 3, ERR_RESOURCE_EXHAUSTED = 8,
                           ERR_INTERNAL = 13 };

struct Buffer {
  size_t struct_size;
  ExtBase* extension_start;
  int32_t dtype;
  void* data;
  int64_t rank;
  int64_t* dims;
};
struct Args {
  size_t struct_size;
  ExtBase* extension_start;
  int64_t size;
  int32_t* types;
  void** args;
};
struct ByteSpan {
  const char* ptr;
  size_t len;
};
struct Array {
  int32_t dtype;
  size_t size;
  void* data;
};
struct Attrs {
  size_t struct_size;
  ExtBase* extension_start;
  int64_t size;
  int32_t* types;
  ByteSpan** names;
  void** attrs;
};
struct CallFrame {
  size_t struct_size;
  ExtBase* extension_start;
  const Api* api;
  Ctx* ctx;
  int32_t stage;
  Args args;
  Args rets;   // same layout as the arguments (result types instead of argument types)
  Attrs attrs;
};
struct ErrorCreateArgs {
  size_t struct_size;
  ExtBase* extension_start;
  const char* message;
  int32_t errc;
};
struct StreamGetArgs {
  size_t struct_size;
  ExtBase* extension_start;
  Ctx* ctx;
  void* stream;   // out
};
struct ApiVersion {
  size_t struct_size;
  ExtBase* extension_start;
  int32_t major_version;
  int32_t minor_version;
};
typedef Error* (*ErrorCreateFn)(ErrorCreateArgs*);
typedef Error* (*StreamGetFn)(StreamGetArgs*);
struct Api {
  size_t struct_size;
  ExtBase* extension_start;
  ApiVersion api_version;
  void* internal_api;
  ErrorCreateFn error_create;
  void* error_get_message;
  void* error_destroy;
  void* handler_register;
  StreamGetFn stream_get;
};

// an XLA error "fn: what" (XLA copies the message)
Error* fail(const CallFrame* f, int32_t code, const char* fn, const char* what) {
  static thread_local char msg[256];
  snprintf(msg, sizeof msg, "%s: %s", fn, what);
  if (!f || !f->api || !f->api->error_create) return nullptr;
  ErrorCreateArgs a{sizeof(ErrorCreateArgs), nullptr, msg, code};
  return f->api->error_create(&a);
}
Error* failk(const CallFrame* f, const char* fn, const char* fmt, int k) {
  static thread_local char what[160];
  snprintf(what, sizeof what, fmt, k);
  return fail(f, ERR_INVALID_ARGUMENT, fn, what);
}

const Buffer* buffer(const Args& a, int k) {
  if (k >= a.size || !a.types || a.types[k] != ARG_BUFFER) return nullptr;
  const Buffer* b = static_cast<const Buffer*>(a.args[k]);
  return (b && b->struct_size >= sizeof(Buffer)) ? b : nullptr;
}

int64_t elements(const Buffer* b) {
  int64_t n = 1;
  for (int64_t d = 0; d < b->rank; ++d) n *= b->dims[d];
  return n;
}

// the step parameters travel as one U8 array attribute "params" holding the
// bytes of an AjStepParams
bool params_attr(const CallFrame* f, AjStepParams* out) {
  const Attrs& at = f->attrs;
  for (int64_t k = 0; k < at.size; ++k) {
    const ByteSpan* nm = at.names[k];
    if (!nm || nm->len != 6 || memcmp(nm->ptr, "params", 6) != 0) continue;
    if (at.types[k] != ATTR_ARRAY) return false;
    const Array* arr = static_cast<const Array*>(at.attrs[k]);
    if (!arr || arr->dtype != DT_U8 || arr->size != sizeof(AjStepParams)) return false;
    memcpy(out, arr->data, sizeof(AjStepParams));
    return true;
  }
  return false;
}

bool frame_ok(const CallFrame* f) {
  return f && f->struct_size >= sizeof(CallFrame) && f->api &&
         f->api->struct_size >= sizeof(Api) && f->args.struct_size >= sizeof(Args) &&
         f->rets.struct_size >= sizeof(Args) && f->attrs.struct_size >= sizeof(Attrs);
}

void* stream_of(const CallFrame* f) {
  if (!f->api->stream_get) return nullptr;
  StreamGetArgs a{sizeof(StreamGetArgs), nullptr, f->ctx, nullptr};
  if (f->api->stream_get(&a) != nullptr) return nullptr;
  return a.stream;
}

const char* status_name(int rc) {
  switch (rc) {
    case AJ_ERR_SHAPE: return "AJ_ERR_SHAPE";
    case AJ_ERR_PARAM: return "AJ_ERR_PARAM";
    case AJ_ERR_WORKSPACE: return "AJ_ERR_WORKSPACE";
    case AJ_ERR_CUDA: return "AJ_ERR_CUDA";
    default: return "AJ_ERR";
  }
}

Error* status(const CallFrame* f, const char* fn, int rc) {
  if (rc == AJ_OK) return nullptr;
  const int32_t code = rc == AJ_ERR_CUDA ? ERR_INTERNAL
                       : rc == AJ_ERR_WORKSPACE ? ERR_RESOURCE_EXHAUSTED
                                                : ERR_INVALID_ARGUMENT;
  static thread_local char what[64];
  snprintf(what, sizeof what, "%s (status %d)", status_name(rc), rc);
  return fail(f, code, fn, what);
}

// field sizes of a grid: u, v (MAC faces or cells) and p
void field_sizes(const AjStepParams& p, int64_t* nu, int64_t* nv, int64_t* np_) {
  const bool mac = p.grid_type == AJ_GRID_MAC;
  *nu = (int64_t)(mac ? p.nx + 1 : p.nx) * p.ny;
  *nv = (int64_t)p.nx * (mac ? p.ny + 1 : p.ny);
  *np_ = (int64_t)p.nx * p.ny;
}

}  // namespace ffi
}  // namespace aj

using namespace aj;
using namespace aj::ffi;

extern "C" {

// aj_step as a custom call.  Arguments: u, v, mask, p_guess (F32; p_guess
// may have 0 elements when the step ignores it), workspace (U8, from
// aj_ffi_prepare).  Results: u_out, v_out, p_out (F32) and, optionally, the
// workspace again (alias it with the workspace argument so that XLA treats
// the scratch as written).  Attribute "params": the AjStepParams bytes.
void* aj_ffi_step(void* frame) {
  const CallFrame* f = static_cast<const CallFrame*>(frame);
  if (!frame_ok(f)) return fail(f, ERR_INVALID_ARGUMENT, "aj_ffi_step", "bad call frame");
  if (f->stage != STAGE_EXECUTE) return nullptr;
  AjStepParams p;
  if (!params_attr(f, &p))
    return failk(f, "aj_ffi_step", "attribute 'params' (u8[%d]) missing",
                 (int)sizeof(AjStepParams));
  const Buffer* in[5];
  for (int k = 0; k < 5; ++k)
    if (!(in[k] = buffer(f->args, k)))
      return failk(f, "aj_ffi_step", "argument %d is not a buffer", k);
  const Buffer* out[3];
  for (int k = 0; k < 3; ++k)
    if (!(out[k] = buffer(f->rets, k)))
      return failk(f, "aj_ffi_step", "result %d is not a buffer", k);
  int64_t nu, nv, np_;
  field_sizes(p, &nu, &nv, &np_);
  const int64_t want_in[4] = {nu, nv, np_, np_}, want_out[3] = {nu, nv, np_};
  for (int k = 0; k < 4; ++k) {
    if (in[k]->dtype != DT_F32)
      return failk(f, "aj_ffi_step", "argument %d must be float32", k);
    const int64_t n = elements(in[k]);
    if (n != want_in[k] && !(k == 3 && n == 0))
      return failk(f, "aj_ffi_step", "argument %d has the wrong size", k);
  }
  for (int k = 0; k < 3; ++k)
    if (out[k]->dtype != DT_F32 || elements(out[k]) != want_out[k])
      return failk(f, "aj_ffi_step", "result %d must be float32 of the field size", k);
  const Buffer* ws = in[4];
  if (f->rets.size >= 4) {
    const Buffer* wo = buffer(f->rets, 3);
    if (!wo) return failk(f, "aj_ffi_step", "result %d is not a buffer", 3);
    ws = wo;   // the aliased workspace (same memory as the argument)
  }
  if (ws->dtype != DT_U8)
    return fail(f, ERR_INVALID_ARGUMENT, "aj_ffi_step", "the workspace must be uint8");
  int rc = aj_check_params(&p);
  if (rc != AJ_OK) return status(f, "aj_step", rc);
  void* st = stream_of(f);
  const float* pg = elements(in[3]) ? static_cast<const float*>(in[3]->data) : nullptr;
  rc = aj_step(&p, static_cast<const float*>(in[0]->data), static_cast<const float*>(in[1]->data),
               static_cast<const float*>(in[2]->data), pg, static_cast<float*>(out[0]->data),
               static_cast<float*>(out[1]->data), static_cast<float*>(out[2]->data), ws->data,
               (size_t)elements(ws), nullptr, st);
  return status(f, "aj_step", rc);
}

// aj_prepare as a custom call: argument mask (F32), sdf (F32, 0 elements for
// none); result: the workspace (U8, aj_workspace_size bytes).  Synchronous,
// like aj_prepare: call it when the geometry changes (the reference rebuilds
// its step at that moment, solver/simulation/flow_control.py:162-194).
void* aj_ffi_prepare(void* frame) {
  const CallFrame* f = static_cast<const CallFrame*>(frame);
  if (!frame_ok(f)) return fail(f, ERR_INVALID_ARGUMENT, "aj_ffi_prepare", "bad call frame");
  if (f->stage != STAGE_EXECUTE) return nullptr;
  AjStepParams p;
  if (!params_attr(f, &p))
    return failk(f, "aj_ffi_prepare", "attribute 'params' (u8[%d]) missing",
                 (int)sizeof(AjStepParams));
  const Buffer* mask = buffer(f->args, 0);
  const Buffer* sdf = buffer(f->args, 1);
  const Buffer* ws = buffer(f->rets, 0);
  if (!mask || !sdf || !ws)
    return fail(f, ERR_INVALID_ARGUMENT, "aj_ffi_prepare", "expects (mask, sdf) -> workspace");
  int64_t nu, nv, np_;
  field_sizes(p, &nu, &nv, &np_);
  if (mask->dtype != DT_F32 || elements(mask) != np_ || sdf->dtype != DT_F32 ||
      (elements(sdf) != 0 && elements(sdf) != np_) || ws->dtype != DT_U8)
    return fail(f, ERR_INVALID_ARGUMENT, "aj_ffi_prepare", "bad buffer types or sizes");
  int rc = aj_check_params(&p);
  if (rc != AJ_OK) return status(f, "aj_prepare", rc);
  const size_t need = aj_workspace_size(&p);
  if ((size_t)elements(ws) < need)
    return status(f, "aj_prepare", AJ_ERR_WORKSPACE);
  const float* s = elements(sdf) ? static_cast<const float*>(sdf->data) : nullptr;
  rc = aj_prepare(&p, static_cast<const float*>(mask->data), s, ws->data, (size_t)elements(ws),
                  stream_of(f));
  return status(f, "aj_prepare", rc);
}

}  // extern "C"
