/*
 * napi_stub.c - a tiny stand-in for Node's Node-API, for testing the addon
 * (caustic-tracer_gb300/napi/caustic_addon.c) without Node.
 *
 * TEST INFRASTRUCTURE. It implements the Node-API calls the addon makes over
 * a minimal value model (undefined, null, booleans, numbers, strings, plain
 * objects, ArrayBuffers, typed arrays, externals, functions) and exports
 * stub_* helpers through which a Python test builds argument values, loads
 * the addon (napi_register_module_v1), calls its functions and reads results
 * and pending exceptions. Values live until stub_env_free, which also runs
 * the finalizers of externals, as Node does when their handles are collected.
 */
#define _GNU_SOURCE
#include <dlfcn.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "node_api_min.h"

enum { K_UNDEF, K_NULL, K_BOOL, K_NUM, K_STR, K_OBJ, K_ABUF, K_TYPED, K_EXT, K_FUNC };

struct napi_value__ {
  int kind;
  double num;
  bool b;
  char* str;
  /* object */
  size_t n, cap;
  char** keys;
  napi_value* vals;
  /* ArrayBuffer */
  void* data;
  size_t bytes;
  int owned;
  /* typed array over `buffer` */
  napi_typedarray_type ttype;
  size_t length, offset;
  napi_value buffer;
  /* external */
  void* ext;
  napi_finalize fin;
  void* hint;
  int finalized;
  /* function */
  napi_callback cb;
  void* cbdata;
  napi_value next; /* all values of the env */
};

struct napi_env__ {
  napi_value all;
  napi_value undef;
  int pending; /* 0 none, 1 Error, 2 TypeError, 3 RangeError */
  char code[96];
  char msg[1024];
  int finalized;
};

struct napi_callback_info__ {
  size_t argc;
  napi_value* argv;
  void* data;
};

static const size_t kElem[] = {1, 1, 1, 2, 2, 4, 4, 4, 8, 8, 8};

static napi_value make(napi_env env, int kind) {
  napi_value v = (napi_value)calloc(1, sizeof *v);
  v->kind = kind;
  v->next = env->all;
  env->all = v;
  return v;
}

/* ---- the Node-API calls ------------------------------------------------- */

napi_status napi_get_cb_info(napi_env env, napi_callback_info cbinfo, size_t* argc, napi_value* argv,
                             napi_value* this_arg, void** data) {
  if (!env || !cbinfo) return napi_invalid_arg;
  if (argc) {
    for (size_t i = 0; i < *argc; i++) argv[i] = i < cbinfo->argc ? cbinfo->argv[i] : env->undef;
    *argc = cbinfo->argc;
  }
  if (this_arg) *this_arg = env->undef;
  if (data) *data = cbinfo->data;
  return napi_ok;
}

napi_status napi_typeof(napi_env env, napi_value value, napi_valuetype* result) {
  if (!env || !value || !result) return napi_invalid_arg;
  switch (value->kind) {
    case K_UNDEF: *result = napi_undefined; break;
    case K_NULL: *result = napi_null; break;
    case K_BOOL: *result = napi_boolean; break;
    case K_NUM: *result = napi_number; break;
    case K_STR: *result = napi_string; break;
    case K_EXT: *result = napi_external; break;
    case K_FUNC: *result = napi_function; break;
    default: *result = napi_object;
  }
  return napi_ok;
}

napi_status napi_get_undefined(napi_env env, napi_value* result) {
  if (!env || !result) return napi_invalid_arg;
  *result = env->undef;
  return napi_ok;
}

static napi_value lookup(napi_value obj, const char* key) {
  for (size_t i = 0; i < obj->n; i++)
    if (strcmp(obj->keys[i], key) == 0) return obj->vals[i];
  return NULL;
}

napi_status napi_get_named_property(napi_env env, napi_value object, const char* utf8name, napi_value* result) {
  if (!env || !object || !utf8name || !result) return napi_invalid_arg;
  if (object->kind != K_OBJ && object->kind != K_TYPED && object->kind != K_ABUF) return napi_object_expected;
  napi_value v = object->kind == K_OBJ ? lookup(object, utf8name) : NULL;
  *result = v ? v : env->undef;
  return napi_ok;
}

napi_status napi_has_named_property(napi_env env, napi_value object, const char* utf8name, bool* result) {
  if (!env || !object || !utf8name || !result) return napi_invalid_arg;
  if (object->kind != K_OBJ && object->kind != K_TYPED && object->kind != K_ABUF) return napi_object_expected;
  *result = object->kind == K_OBJ && lookup(object, utf8name) != NULL;
  return napi_ok;
}

napi_status napi_get_value_double(napi_env env, napi_value value, double* result) {
  if (!env || !value || !result) return napi_invalid_arg;
  if (value->kind != K_NUM) return napi_number_expected;
  *result = value->num;
  return napi_ok;
}

napi_status napi_get_value_bool(napi_env env, napi_value value, bool* result) {
  if (!env || !value || !result) return napi_invalid_arg;
  if (value->kind != K_BOOL) return napi_boolean_expected;
  *result = value->b;
  return napi_ok;
}

napi_status napi_get_value_string_utf8(napi_env env, napi_value value, char* buf, size_t bufsize, size_t* result) {
  if (!env || !value) return napi_invalid_arg;
  if (value->kind != K_STR) return napi_string_expected;
  size_t len = strlen(value->str);
  if (!buf) {
    if (!result) return napi_invalid_arg;
    *result = len;
    return napi_ok;
  }
  size_t copy = bufsize ? (len < bufsize - 1 ? len : bufsize - 1) : 0;
  if (bufsize) {
    memcpy(buf, value->str, copy);
    buf[copy] = 0;
  }
  if (result) *result = copy;
  return napi_ok;
}

napi_status napi_is_typedarray(napi_env env, napi_value value, bool* result) {
  if (!env || !value || !result) return napi_invalid_arg;
  *result = value->kind == K_TYPED;
  return napi_ok;
}

napi_status napi_get_typedarray_info(napi_env env, napi_value typedarray, napi_typedarray_type* type, size_t* length,
                                     void** data, napi_value* arraybuffer, size_t* byte_offset) {
  if (!env || !typedarray) return napi_invalid_arg;
  if (typedarray->kind != K_TYPED) return napi_invalid_arg;
  if (type) *type = typedarray->ttype;
  if (length) *length = typedarray->length;
  if (data) *data = (char*)typedarray->buffer->data + typedarray->offset;
  if (arraybuffer) *arraybuffer = typedarray->buffer;
  if (byte_offset) *byte_offset = typedarray->offset;
  return napi_ok;
}

napi_status napi_create_arraybuffer(napi_env env, size_t byte_length, void** data, napi_value* result) {
  if (!env || !result) return napi_invalid_arg;
  napi_value v = make(env, K_ABUF);
  v->data = calloc(byte_length ? byte_length : 1, 1); /* zero-filled, as a new ArrayBuffer */
  if (!v->data) return napi_generic_failure;
  v->bytes = byte_length;
  v->owned = 1;
  if (data) *data = v->data;
  *result = v;
  return napi_ok;
}

napi_status napi_create_typedarray(napi_env env, napi_typedarray_type type, size_t length, napi_value arraybuffer,
                                   size_t byte_offset, napi_value* result) {
  if (!env || !arraybuffer || !result || (int)type < 0 || (int)type > (int)napi_biguint64_array)
    return napi_invalid_arg;
  if (arraybuffer->kind != K_ABUF) return napi_invalid_arg;
  const size_t e = kElem[type];
  if (byte_offset % e || byte_offset + length * e > arraybuffer->bytes) return napi_invalid_arg;
  napi_value v = make(env, K_TYPED);
  v->ttype = type;
  v->length = length;
  v->offset = byte_offset;
  v->buffer = arraybuffer;
  *result = v;
  return napi_ok;
}

napi_status napi_create_external(napi_env env, void* data, napi_finalize finalize_cb, void* finalize_hint,
                                 napi_value* result) {
  if (!env || !result) return napi_invalid_arg;
  napi_value v = make(env, K_EXT);
  v->ext = data;
  v->fin = finalize_cb;
  v->hint = finalize_hint;
  *result = v;
  return napi_ok;
}

napi_status napi_get_value_external(napi_env env, napi_value value, void** result) {
  if (!env || !value || !result) return napi_invalid_arg;
  if (value->kind != K_EXT) return napi_invalid_arg;
  *result = value->ext;
  return napi_ok;
}

static napi_status throw_kind(napi_env env, int kind, const char* code, const char* msg) {
  if (!env || !msg) return napi_invalid_arg;
  if (env->pending) return napi_pending_exception;
  env->pending = kind;
  snprintf(env->code, sizeof env->code, "%s", code ? code : "");
  snprintf(env->msg, sizeof env->msg, "%s", msg);
  return napi_ok;
}

napi_status napi_throw_error(napi_env env, const char* code, const char* msg) { return throw_kind(env, 1, code, msg); }
napi_status napi_throw_type_error(napi_env env, const char* code, const char* msg) {
  return throw_kind(env, 2, code, msg);
}
napi_status napi_throw_range_error(napi_env env, const char* code, const char* msg) {
  return throw_kind(env, 3, code, msg);
}

napi_status napi_is_exception_pending(napi_env env, bool* result) {
  if (!env || !result) return napi_invalid_arg;
  *result = env->pending != 0;
  return napi_ok;
}

static int set_prop(napi_value obj, const char* key, napi_value val) {
  for (size_t i = 0; i < obj->n; i++)
    if (strcmp(obj->keys[i], key) == 0) {
      obj->vals[i] = val;
      return 1;
    }
  if (obj->n == obj->cap) {
    size_t cap = obj->cap ? 2 * obj->cap : 8;
    char** k = (char**)realloc(obj->keys, cap * sizeof *k);
    if (!k) return 0;
    obj->keys = k;
    napi_value* v = (napi_value*)realloc(obj->vals, cap * sizeof *v);
    if (!v) return 0;
    obj->vals = v;
    obj->cap = cap;
  }
  obj->keys[obj->n] = strdup(key);
  obj->vals[obj->n++] = val;
  return 1;
}

napi_status napi_define_properties(napi_env env, napi_value object, size_t property_count,
                                   const napi_property_descriptor* properties) {
  if (!env || !object || (property_count && !properties)) return napi_invalid_arg;
  if (object->kind != K_OBJ) return napi_object_expected;
  for (size_t i = 0; i < property_count; i++) {
    const napi_property_descriptor* d = &properties[i];
    if (!d->utf8name) return napi_name_expected;
    napi_value v = d->value;
    if (d->method) {
      v = make(env, K_FUNC);
      v->cb = d->method;
      v->cbdata = d->data;
    }
    if (!v || !set_prop(object, d->utf8name, v)) return napi_generic_failure;
  }
  return napi_ok;
}

/* ---- helpers for the test ----------------------------------------------- */

napi_env stub_env_new(void) {
  napi_env env = (napi_env)calloc(1, sizeof *env);
  env->undef = make(env, K_UNDEF);
  return env;
}

/* Runs every external's finalizer that has not run yet (as garbage collection would). */
int stub_collect(napi_env env) {
  int n = 0;
  for (napi_value v = env->all; v; v = v->next)
    if (v->kind == K_EXT && !v->finalized) {
      v->finalized = 1;
      if (v->fin) v->fin(env, v->ext, v->hint);
      n++;
    }
  env->finalized += n;
  return n;
}

void stub_env_free(napi_env env) {
  stub_collect(env);
  napi_value v = env->all;
  while (v) {
    napi_value next = v->next;
    if (v->owned) free(v->data);
    free(v->str);
    for (size_t i = 0; i < v->n; i++) free(v->keys[i]);
    free(v->keys);
    free(v->vals);
    free(v);
    v = next;
  }
  free(env);
}

napi_value stub_undefined(napi_env env) { return env->undef; }
napi_value stub_null(napi_env env) { return make(env, K_NULL); }
napi_value stub_bool(napi_env env, int b) {
  napi_value v = make(env, K_BOOL);
  v->b = b != 0;
  return v;
}
napi_value stub_number(napi_env env, double d) {
  napi_value v = make(env, K_NUM);
  v->num = d;
  return v;
}
napi_value stub_string(napi_env env, const char* s) {
  napi_value v = make(env, K_STR);
  v->str = strdup(s);
  return v;
}
napi_value stub_object(napi_env env) { return make(env, K_OBJ); }
int stub_set(napi_env env, napi_value obj, const char* key, napi_value val) {
  (void)env;
  return obj->kind == K_OBJ && set_prop(obj, key, val);
}

/* A typed array over memory the caller owns (kept alive by the caller). */
napi_value stub_typed(napi_env env, int type, void* data, size_t length) {
  napi_value buf = make(env, K_ABUF);
  buf->data = data;
  buf->bytes = length * kElem[type];
  napi_value v = make(env, K_TYPED);
  v->ttype = (napi_typedarray_type)type;
  v->length = length;
  v->buffer = buf;
  return v;
}

int stub_kind(napi_value v) { return v ? v->kind : -1; }
double stub_number_of(napi_value v) { return v && v->kind == K_NUM ? v->num : 0.0; }
int stub_typed_info(napi_value v, int* type, void** data, size_t* length) {
  if (!v || v->kind != K_TYPED) return 0;
  *type = (int)v->ttype;
  *data = (char*)v->buffer->data + v->offset;
  *length = v->length;
  return 1;
}
int stub_finalized(napi_env env) { return env->finalized; }

/* Loads an addon as Node does: dlopen, then napi_register_module_v1(env, exports).
 * RTLD_DEEPBIND makes the addon resolve its own library dependencies first. */
napi_value stub_load(napi_env env, const char* path, char* err, size_t cap) {
  void* h = dlopen(path, RTLD_NOW | RTLD_LOCAL | RTLD_DEEPBIND);
  if (!h) {
    snprintf(err, cap, "%s", dlerror());
    return NULL;
  }
  typedef napi_value (*init_fn)(napi_env, napi_value);
  init_fn init = (init_fn)dlsym(h, "napi_register_module_v1");
  if (!init) {
    snprintf(err, cap, "napi_register_module_v1 not exported by %s", path);
    return NULL;
  }
  napi_value exports = make(env, K_OBJ);
  napi_value r = init(env, exports);
  if (!r) snprintf(err, cap, "module init returned NULL: %s", env->msg);
  return r;
}

/* Calls exports[name](argv...); returns its result (undefined for NULL). */
napi_value stub_call(napi_env env, napi_value exports, const char* name, size_t argc, napi_value* argv) {
  napi_value f = exports && exports->kind == K_OBJ ? lookup(exports, name) : NULL;
  if (!f || f->kind != K_FUNC) {
    throw_kind(env, 2, "ERR_NOT_A_FUNCTION", name);
    return env->undef;
  }
  struct napi_callback_info__ info = {argc, argv, f->cbdata};
  napi_value r = f->cb(env, &info);
  return r ? r : env->undef;
}

/* 0 when nothing is pending; else the kind (1 Error, 2 TypeError, 3 RangeError), copied out and cleared. */
int stub_take_exception(napi_env env, char* code, size_t code_cap, char* msg, size_t msg_cap) {
  int k = env->pending;
  if (!k) return 0;
  snprintf(code, code_cap, "%s", env->code);
  snprintf(msg, msg_cap, "%s", env->msg);
  env->pending = 0;
  return k;
}
