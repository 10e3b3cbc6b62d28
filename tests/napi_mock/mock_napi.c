/* TEST INFRASTRUCTURE: a minimal N-API runtime for running the libwt addon
 * (f1-wind-tunnel_gb300/napi/wt_napi.c) without Node.  Values are tagged host
 * structs; the program registers the module, then calls the exported functions
 * named on its command line the way engine.ts would, and prints one line per
 * call: "<name> ok <number>" or "<name> threw <message>". */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "node_api.h"

enum { V_NUM, V_EXT, V_TYPED, V_STR };
struct napi_value__ {
  int kind;
  double num;
  void* ptr;
  size_t len;
  napi_typedarray_type type;
  const char* str;
};
struct napi_env__ {
  char error[1024];
  int thrown;
  napi_property_descriptor props[64];
  size_t nprops;
};
struct napi_callback_info__ {
  size_t argc;
  napi_value argv[8];
};

napi_status napi_get_cb_info(napi_env env, napi_callback_info cb, size_t* argc, napi_value* argv, napi_value* t,
                             void** d) {
  (void)env; (void)t; (void)d;
  size_t n = *argc < cb->argc ? *argc : cb->argc;
  for (size_t i = 0; i < n; i++) argv[i] = cb->argv[i];
  *argc = cb->argc;
  return napi_ok;
}
napi_status napi_get_value_double(napi_env env, napi_value v, double* r) {
  (void)env;
  if (!v || v->kind != V_NUM) return napi_number_expected;
  *r = v->num;
  return napi_ok;
}
napi_status napi_get_value_int32(napi_env env, napi_value v, int32_t* r) {
  (void)env;
  if (!v || v->kind != V_NUM) return napi_number_expected;
  *r = (int32_t)v->num;
  return napi_ok;
}
napi_status napi_get_value_bool(napi_env env, napi_value v, bool* r) {
  (void)env;
  if (!v || v->kind != V_NUM) return napi_boolean_expected;
  *r = v->num != 0.0;
  return napi_ok;
}
napi_status napi_get_value_external(napi_env env, napi_value v, void** r) {
  (void)env;
  if (!v || v->kind != V_EXT) return napi_invalid_arg;
  *r = v->ptr;
  return napi_ok;
}
napi_status napi_get_value_string_utf8(napi_env env, napi_value v, char* buf, size_t size, size_t* r) {
  (void)env;
  if (!v || v->kind != V_STR) return napi_string_expected;
  snprintf(buf, size, "%s", v->str);
  *r = strlen(buf);
  return napi_ok;
}
napi_status napi_get_typedarray_info(napi_env env, napi_value v, napi_typedarray_type* t, size_t* len, void** data,
                                     napi_value* ab, size_t* off) {
  (void)env; (void)ab; (void)off;
  if (!v || v->kind != V_TYPED) return napi_invalid_arg;
  if (t) *t = v->type;
  if (len) *len = v->len;
  if (data) *data = v->ptr;
  return napi_ok;
}
napi_status napi_create_external(napi_env env, void* data, napi_finalize f, void* hint, napi_value* r) {
  (void)env; (void)f; (void)hint;
  *r = calloc(1, sizeof(struct napi_value__));
  (*r)->kind = V_EXT;
  (*r)->ptr = data;
  return napi_ok;
}
napi_status napi_create_double(napi_env env, double d, napi_value* r) {
  (void)env;
  *r = calloc(1, sizeof(struct napi_value__));
  (*r)->kind = V_NUM;
  (*r)->num = d;
  return napi_ok;
}
napi_status napi_throw_error(napi_env env, const char* code, const char* msg) {
  (void)code;
  env->thrown = 1;
  snprintf(env->error, sizeof(env->error), "%s", msg);
  return napi_ok;
}
napi_status napi_define_properties(napi_env env, napi_value o, size_t n, const napi_property_descriptor* p) {
  (void)o;
  for (size_t i = 0; i < n && env->nprops < 64; i++) env->props[env->nprops++] = p[i];
  return napi_ok;
}

static napi_value num(double d) {
  napi_value v = calloc(1, sizeof(struct napi_value__));
  v->kind = V_NUM;
  v->num = d;
  return v;
}
static napi_value f32(const float* p, size_t n) {
  napi_value v = calloc(1, sizeof(struct napi_value__));
  v->kind = V_TYPED;
  v->ptr = (void*)p;
  v->len = n;
  v->type = napi_float32_array;
  return v;
}
static napi_value ext(void* p) {
  napi_value v = calloc(1, sizeof(struct napi_value__));
  v->kind = V_EXT;
  v->ptr = p;
  return v;
}

static napi_callback find(napi_env env, const char* name) {
  for (size_t i = 0; i < env->nprops; i++)
    if (!strcmp(env->props[i].utf8name, name)) return env->props[i].method;
  return NULL;
}

static void report(napi_env env, const char* name, napi_value r) {
  if (env->thrown) printf("%s threw %s\n", name, env->error);
  else printf("%s ok %g\n", name, r && r->kind == V_NUM ? r->num : 0.0);
  env->thrown = 0;
}

int main(void) {
  struct napi_env__ env;
  memset(&env, 0, sizeof(env));
  napi_register_module_v1(&env, NULL);
  printf("exports %zu\n", env.nprops);
  for (size_t i = 0; i < env.nprops; i++) printf("export %s\n", env.props[i].utf8name);
  /* create(16, 8, 8, [0, 0, 0, 0.1]): a context where a GB300 is present, a thrown libwt error elsewhere */
  float origin[4] = {0.0f, 0.0f, 0.0f, 0.1f};
  struct napi_callback_info__ ci = {4, {num(16), num(8), num(8), f32(origin, 4)}};
  napi_value h = find(&env, "create")(&env, &ci);
  report(&env, "create", NULL);
  /* a malformed create: no origin array */
  struct napi_callback_info__ bad = {3, {num(16), num(8), num(8)}};
  find(&env, "create")(&env, &bad);
  report(&env, "create_bad", NULL);
  /* step with an odd count on the handle (or on no context): libwt refuses it */
  struct napi_callback_info__ st = {2, {h ? h : ext(NULL), num(3)}};
  find(&env, "step")(&env, &st);
  report(&env, "step_odd", NULL);
  if (h) {
    struct napi_callback_info__ s2 = {2, {h, num(8)}};
    find(&env, "step")(&env, &s2);
    report(&env, "step", NULL);
    int32_t raw[12];
    napi_value ra = calloc(1, sizeof(struct napi_value__));
    ra->kind = V_TYPED; ra->ptr = raw; ra->len = 12; ra->type = napi_int32_array;
    struct napi_callback_info__ rf = {2, {h, ra}};
    napi_value steps = find(&env, "readForces")(&env, &rf);
    report(&env, "readForces", steps);
  }
  return 0;
}
