// rtc.cu -- user right-hand sides compiled at run time with NVRTC.
//
// The reference's problems take any Julia function f!(du, u, p, t)
// (ODEFunction, test/qa/qa.jl:84); a precompiled kernel library can only
// offer built-in models.  This file closes the gap: a caller registers the
// body of f (and optionally of its Jacobian) as CUDA C++ source
// (gbde_model_register), and the first solve of that model with a given
// algorithm and precision compiles the library's own step kernels around it --
// the same headers as the precompiled kernels (integrate_all, the steppers,
// the controller, the dense output) -- with NVRTC for sm_103a, loads the cubin
// as a context-independent library and launches it like a built-in kernel.
// Without a user Jacobian, Rosenbrock methods differentiate f by forward-mode
// dual numbers (dual.cuh), the counterpart of the reference's ForwardDiff
// default (AutoForwardDiff, qa.jl:12).
//
// NVRTC is opened with dlopen at the first compile, so the library loads
// (and every built-in model works) where NVRTC is absent.
#include <dlfcn.h>
#include <nvrtc.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/gbde.h"
#include "launch.h"

namespace gbde {
int set_thread_error(int code, const char* msg);
}

using namespace gbde;

namespace {

// kRtcHeaders[]: {include name, text} of every header the runtime-compiled
// source includes, embedded at build time (build.py writes rtc_headers.inc).
struct RtcHeader {
  const char* name;
  const char* text;
};
#include "rtc_headers.inc"

// ------------------------------------------------------------------ NVRTC
struct Nvrtc {
  bool ok = false;
  std::string why;
  nvrtcResult (*create)(nvrtcProgram*, const char*, const char*, int, const char* const*,
                        const char* const*) = nullptr;
  nvrtcResult (*compile)(nvrtcProgram, int, const char* const*) = nullptr;
  nvrtcResult (*log_size)(nvrtcProgram, size_t*) = nullptr;
  nvrtcResult (*log)(nvrtcProgram, char*) = nullptr;
  nvrtcResult (*cubin_size)(nvrtcProgram, size_t*) = nullptr;
  nvrtcResult (*cubin)(nvrtcProgram, char*) = nullptr;
  nvrtcResult (*destroy)(nvrtcProgram*) = nullptr;
  const char* (*err_str)(nvrtcResult) = nullptr;
};

Nvrtc load_nvrtc() {
  Nvrtc n;
  void* h = nullptr;
  std::vector<std::string> names = {"libnvrtc.so.13", "libnvrtc.so"};
  if (const char* home = std::getenv("CUDA_HOME")) {
    names.push_back(std::string(home) + "/lib64/libnvrtc.so.13");
    names.push_back(std::string(home) + "/lib64/libnvrtc.so");
  }
  for (const auto& nm : names)
    if ((h = dlopen(nm.c_str(), RTLD_NOW | RTLD_LOCAL)) != nullptr) break;
  if (!h) {
    n.why = "NVRTC (libnvrtc.so.13) not found: user models need the CUDA toolkit's NVRTC";
    return n;
  }
#define GBDE_SYM(field, name)                                            \
  n.field = reinterpret_cast<decltype(n.field)>(dlsym(h, name));         \
  if (!n.field) {                                                        \
    n.why = std::string("NVRTC symbol ") + name + " missing";            \
    return n;                                                            \
  }
  GBDE_SYM(create, "nvrtcCreateProgram")
  GBDE_SYM(compile, "nvrtcCompileProgram")
  GBDE_SYM(log_size, "nvrtcGetProgramLogSize")
  GBDE_SYM(log, "nvrtcGetProgramLog")
  GBDE_SYM(cubin_size, "nvrtcGetCUBINSize")
  GBDE_SYM(cubin, "nvrtcGetCUBIN")
  GBDE_SYM(destroy, "nvrtcDestroyProgram")
  GBDE_SYM(err_str, "nvrtcGetErrorString")
#undef GBDE_SYM
  n.ok = true;
  return n;
}

Nvrtc& nvrtc() {
  static Nvrtc n = load_nvrtc();
  return n;
}

// --------------------------------------------------------------- registry
struct UserModelDef {
  std::string name, f_body, jac_body, g_body;  // g_body: diagonal noise (SDE models)
  int n, np;
};

// A registered callback: a leaf (GBDE_CB_CONTINUOUS / _DISCRETE / _VECTOR,
// len conditions for a vector one) or a set (kind 0) of earlier ids.
struct CallbackDef {
  int kind = 0, len = 1;
  int save = 0;             // GBDE_SAVE_BEFORE | GBDE_SAVE_AFTER
  bool has_affect = false;  // an affect or terminate (the state is modified)
  std::string condition, affect;
  std::vector<int> members;
};

struct Compiled {
  std::vector<char> cubin;
  cudaLibrary_t lib = nullptr;
  cudaKernel_t step = nullptr, init = nullptr;
};

using Key = std::tuple<int, int, int, int>;  // (model, alg, precision, callback)

std::mutex g_mu;
std::vector<UserModelDef> g_models;        // id = GBDE_MODEL_USER_BASE + index
std::vector<CallbackDef> g_callbacks;      // id = index + 1
std::map<Key, Compiled> g_compiled;

const CallbackDef* find_callback(int id) {
  return (id >= 1 && id <= (int)g_callbacks.size()) ? &g_callbacks[id - 1] : nullptr;
}

// The leaves of a callback in order, sets expanded (members always have
// smaller ids than their set, so this ends).
void flatten_callback(const CallbackDef* cb, std::vector<const CallbackDef*>& out) {
  if (cb->kind != 0) {
    out.push_back(cb);
    return;
  }
  for (int id : cb->members) flatten_callback(find_callback(id), out);
}

// UserCallback for the driver's interface (solver.cuh): the continuous
// conditions of every ContinuousCallback (one) and VectorContinuousCallback
// (len) in order, and the discrete callbacks in order; the event saves of
// each (save_c / save_d: GBDE_SAVE_* bits; a continuous callback without an
// affect saves nothing after it, as the reference saves only a modified u).
std::string callback_source(const CallbackDef* cb) {
  std::vector<const CallbackDef*> leaves;
  flatten_callback(cb, leaves);
  const std::string args = "const double* u, double t, const double* p";
  const std::string margs = "double* u, double t, const double* p, bool& terminate";
  std::string s, conds, aff_c, cond_d, aff_d, save_c, save_d;
  int nc = 0, nd = 0, saves = 0;
  for (size_t q = 0; q < leaves.size(); ++q) {
    const CallbackDef* l = leaves[q];
    const std::string tag = std::to_string(q);
    const std::string cond_line = "#line 1 \"callback" + tag + ":condition\"\n";
    const std::string aff_line = "#line 1 \"callback" + tag + ":affect\"\n";
    if (l->kind == GBDE_CB_DISCRETE) {
      s += "  __device__ static bool cond_d" + tag + "(" + args + ") {\n    double g = 0.0;\n" +
           cond_line + l->condition + "\n    return g != 0.0;\n  }\n";
      s += "  __device__ static void aff_d" + tag + "(" + margs + ") {\n" + aff_line + l->affect +
           "\n  }\n";
      cond_d += "    case " + std::to_string(nd) + ": return cond_d" + tag + "(u, t, p);\n";
      aff_d += "    case " + std::to_string(nd) + ": aff_d" + tag + "(u, t, p, terminate); return;\n";
      save_d += "    case " + std::to_string(nd) + ": return " + std::to_string(l->save) + ";\n";
      saves |= l->save;
      ++nd;
      continue;
    }
    const int sv = l->save & (l->has_affect ? (GBDE_SAVE_BEFORE | GBDE_SAVE_AFTER) : GBDE_SAVE_BEFORE);
    save_c += "    if (idx < " + std::to_string(nc + l->len) + ") return " + std::to_string(sv) + ";\n";
    saves |= sv;
    const bool vec = l->kind == GBDE_CB_VECTOR;
    s += "  __device__ static void cond_c" + tag + "(" + args + ", double* out) {\n" +
         (vec ? "" : "    double g = 0.0;\n") + cond_line + l->condition +
         (vec ? "\n  }\n" : "\n    out[0] = g;\n  }\n");
    s += "  __device__ static void aff_c" + tag + "(int idx, " + margs + ") {\n    (void)idx;\n" +
         aff_line + l->affect + "\n  }\n";
    conds += "    cond_c" + tag + "(u, t, p, g + " + std::to_string(nc) + ");\n";
    aff_c += "    if (idx < " + std::to_string(nc + l->len) + ") { aff_c" + tag + "(idx - " +
             std::to_string(nc) + ", u, t, p, terminate); return; }\n";
    nc += l->len;
  }
  return "struct UserCallback {\n  static constexpr int NC = " + std::to_string(nc) +
         ", ND = " + std::to_string(nd) + ", SAVES = " + std::to_string(saves) + ";\n" + s +
         "  __device__ static int save_c(int idx) {\n" + save_c + "    return 0;\n  }\n" +
         "  __device__ static int save_d(int k) {\n    switch (k) {\n" + save_d +
         "    }\n    return 0;\n  }\n" +
         "  __device__ static void conditions(" + args + ", double* g) {\n" + conds + "  }\n" +
         "  __device__ static void affect_c(int idx, " + margs + ") {\n" + aff_c + "  }\n" +
         "  __device__ static bool condition_d(int k, " + args + ") {\n    switch (k) {\n" +
         cond_d + "    }\n    return false;\n  }\n" +
         "  __device__ static void affect_d(int k, " + margs + ") {\n    switch (k) {\n" + aff_d +
         "    }\n  }\n};\ntypedef UserCallback GbdeRtcCallback;\n";
}

// Built-in models a runtime-compiled kernel (with a callback) can use.
const char* builtin_model(int id) {
  switch (id) {
    case GBDE_MODEL_LINEAR: return "Linear";
    case GBDE_MODEL_LORENZ: return "Lorenz";
    case GBDE_MODEL_ROBERTSON: return "Robertson";
    case GBDE_MODEL_LOTKA_VOLTERRA: return "LotkaVolterra";
  }
  return nullptr;
}

const UserModelDef* find_model(int id) {
  const int k = id - GBDE_MODEL_USER_BASE;
  return (k >= 0 && k < (int)g_models.size()) ? &g_models[k] : nullptr;
}

const char* prec_type(int precision) {
  return precision == GBDE_PREC_MIXED ? "float" : (precision == GBDE_PREC_F32X2 ? "ff" : "double");
}

// The stepper type the precompiled dispatch (k_explicit.cu, k_rosenbrock.cu)
// uses for this algorithm and precision.
std::string alg_type(int alg, int precision) {
  const std::string T = prec_type(precision);
  if ((alg == GBDE_ALG_EM || alg == GBDE_ALG_SOSRI || alg == GBDE_ALG_SRIW1) &&
      precision == GBDE_PREC_F32X2)
    return "";
  switch (alg) {
    case GBDE_ALG_EM: return "em";
    case GBDE_ALG_SOSRI: return "sri<tab::SosriTab, GBDE_ALG_SOSRI>";
    case GBDE_ALG_SRIW1: return "sri<tab::Sriw1Tab, GBDE_ALG_SRIW1>";
    case GBDE_ALG_TSIT5: return "Tsit5A<GbdeRtcModel, " + T + ">";
    case GBDE_ALG_VERN7: return "Vern7A<GbdeRtcModel, " + T + ">";
    case GBDE_ALG_ROSENBROCK23: return "Ros23A<GbdeRtcModel, " + T + ">";
    case GBDE_ALG_RODAS5:
      return precision == GBDE_PREC_F32X2 ? "RodasFF<GbdeRtcModel, Rodas5Tag>"
                                          : "RodasAlg<GbdeRtcModel, " + T + ", Rodas5Tag>";
    case GBDE_ALG_RODAS5P:
      return precision == GBDE_PREC_F32X2 ? "RodasFF<GbdeRtcModel, Rodas5PTag>"
                                          : "RodasAlg<GbdeRtcModel, " + T + ", Rodas5PTag>";
    case GBDE_ALG_AUTOTSIT5_ROSENBROCK23:
      if (precision == GBDE_PREC_F32X2) return "";
      return "AutoSwitchAlg<GbdeRtcModel, " + T + ", Ros23Alg<GbdeRtcModel, " + T + ">>";
    case GBDE_ALG_AUTOTSIT5_RODAS5:
      if (precision == GBDE_PREC_F32X2) return "";
      return "AutoSwitchAlg<GbdeRtcModel, " + T + ", RodasAlg<GbdeRtcModel, " + T +
             ", Rodas5Tag>>";
  }
  return "";
}

// The runtime-compiled translation unit: fixed-width types (no C library
// under NVRTC), the library's headers, the model (the user's, or a built-in
// one when only the callback is user source), the callback, and two
// extern "C" kernels -- the step kernel and the initial-dt pre-pass --
// instantiated as the precompiled ones are.
std::string make_source(const UserModelDef* m, int model, const CallbackDef* cb, int alg,
                        int precision) {
  const bool mixed = precision != GBDE_PREC_FP64;
  std::string s;
  s += "typedef signed char int8_t; typedef short int16_t; typedef int int32_t;\n"
       "typedef long long int64_t; typedef unsigned char uint8_t;\n"
       "typedef unsigned short uint16_t; typedef unsigned int uint32_t;\n"
       "typedef unsigned long long uint64_t; typedef unsigned long size_t;\n"
       "#include \"solver.cuh\"\n#include \"explicit_rk.cuh\"\n#include \"rosenbrock.cuh\"\n"
       "#include \"rodas_ff.cuh\"\n#include \"tsit5_ff.cuh\"\n#include \"vern7_ff.cuh\"\n#include \"ros23_ff.cuh\"\n#include \"dual.cuh\"\n#include \"sde.cuh\"\n#include \"autoswitch.cuh\"\nnamespace gbde {\n";
  char buf[256];
  if (m) {
    s += "struct UserModel {\n";
    std::snprintf(buf, sizeof(buf),
                  "  static constexpr int N = %d, NP = %d, ID = %d, F_FLOPS = 0;\n", m->n, m->np,
                  model);
    s += buf;
    s += "  template <class T> __device__ static void f(T* du, const T* u, const T* p) {\n";
    s += "#line 1 \"" + m->name + ":f\"\n";
    s += m->f_body;
    s += "\n  }\n  template <class T> __device__ static void jac(T (*J)[N], const T* u, const T* p) {\n";
    if (m->jac_body.empty()) {
      s += "    dual_jacobian<UserModel, T>(J, u, p);\n";
    } else {
      s += "#line 1 \"" + m->name + ":jac\"\n";
      s += m->jac_body;
      s += "\n";
    }
    s += "  }\n";
    if (!m->g_body.empty()) {
      s += "  template <class T> __device__ static void g(T* g, const T* u, const T* p) {\n";
      s += "#line 1 \"" + m->name + ":g\"\n";
      s += m->g_body;
      s += "\n  }\n";
    }
    s += "  __device__ static void features(const double*, const double*, double, float* f) {\n"
         "    for (int i = 0; i < 8; ++i) f[i] = 0.0f;\n  }\n};\n"
         "typedef UserModel GbdeRtcModel;\n";
  } else {
    s += std::string("typedef ") + builtin_model(model) + " GbdeRtcModel;\n";
  }
  if (cb) {
    s += callback_source(cb);
  } else {
    s += "typedef NoCallback GbdeRtcCallback;\n";
  }
  s += "}  // namespace gbde\nusing namespace gbde;\n";
  const std::string at = alg_type(alg, precision);
  s += std::string("typedef ") + prec_type(precision) + " GbdeRtcT;\n";
  if (at == "em" || at.rfind("sri<", 0) == 0) {
    // SDE methods: the library's EM / SRI drivers around the user's f and g;
    // no initial-dt pre-pass (an empty kernel keeps the loader's interface)
    const std::string body =
        at == "em" ? std::string("em_all<GbdeRtcModel, GbdeRtcT>(a);")
                   : "sri_all<GbdeRtcModel, GbdeRtcT, " + std::string(mixed ? "true" : "false") +
                         ", " + at.substr(4, at.size() - 5) + ">(a);";
    s += "extern \"C\" __global__ void __launch_bounds__(128) gbde_rtc_step(const KArgs a) {\n  " +
         body + "\n}\n"
         "extern \"C\" __global__ void gbde_rtc_init_dt(const KArgs, double*) {}\n";
    return s;
  }
  s += "typedef " + at + " GbdeRtcAlg;\n";
  s += "extern \"C\" __global__ void __launch_bounds__(128) gbde_rtc_step(const KArgs a) {\n"
       "  integrate_all<GbdeRtcAlg, GbdeRtcModel, GbdeRtcT, ";
  s += mixed ? "true" : "false";
  s += ", GbdeRtcCallback>(a);\n}\n"
       "extern \"C\" __global__ void __launch_bounds__(128) gbde_rtc_init_dt(const KArgs a, "
       "double* out) {\n  init_dt_all<GbdeRtcAlg, GbdeRtcModel, GbdeRtcT>(a, out);\n}\n";
  return s;
}

int fail(int code, const std::string& msg) { return set_thread_error(code, msg.c_str()); }

// NVRTC compile of one (model, algorithm, precision, callback); g_mu held.
int compile_locked(int id, int alg, int precision, int callback, Compiled** out) {
  const Key key = std::make_tuple(id, alg, precision, callback);
  auto it = g_compiled.find(key);
  if (it != g_compiled.end()) {
    *out = &it->second;
    return GBDE_OK;
  }
  const UserModelDef* m = find_model(id);
  if (!m && !builtin_model(id))
    return fail(GBDE_ERR_INVALID, "model " + std::to_string(id) +
                                      " cannot be compiled at run time (unknown user model, or a "
                                      "built-in model without one-thread kernels)");
  const CallbackDef* cb = nullptr;
  if (callback != 0 && !(cb = find_callback(callback)))
    return fail(GBDE_ERR_INVALID, "unknown callback id " + std::to_string(callback));
  if (cb) {
    std::vector<const CallbackDef*> leaves;
    flatten_callback(cb, leaves);
    int nc = 0;
    for (const CallbackDef* l : leaves) nc += l->kind == GBDE_CB_DISCRETE ? 0 : l->len;
    if (nc > GBDE_MAX_CB_CONDITIONS)
      return fail(GBDE_ERR_INVALID, "the callback set carries " + std::to_string(nc) +
                                        " continuous conditions (at most " +
                                        std::to_string(GBDE_MAX_CB_CONDITIONS) + ")");
  }
  if (alg_type(alg, precision).empty())
    return fail(GBDE_ERR_UNSUPPORTED,
                "runtime-compiled kernels run Tsit5, Vern7, Rosenbrock23, Rodas5 and Rodas5P, "
                "the AutoTsit5 composites in FP64 or mixed precision, and EM, SOSRI and SRIW1 "
                "in FP64 or mixed precision");
  const bool sde = alg == GBDE_ALG_EM || alg == GBDE_ALG_SOSRI || alg == GBDE_ALG_SRIW1;
  if (sde && (cb || !m || m->g_body.empty()))
    return fail(GBDE_ERR_UNSUPPORTED,
                "SDE methods need a user model registered with its noise term "
                "(gbde_sde_model_register), without a callback");
  Nvrtc& nv = nvrtc();
  if (!nv.ok) return fail(GBDE_ERR_UNSUPPORTED, nv.why);
  const std::string src = make_source(m, id, cb, alg, precision);
  const std::string label = m ? m->name : std::string(builtin_model(id));
  std::vector<const char*> hnames, htexts;
  for (const RtcHeader& h : kRtcHeaders) {
    hnames.push_back(h.name);
    htexts.push_back(h.text);
  }
  nvrtcProgram prog = nullptr;
  nvrtcResult r = nv.create(&prog, src.c_str(), (label + ".cu").c_str(), (int)hnames.size(),
                            htexts.data(), hnames.data());
  if (r != NVRTC_SUCCESS) return fail(GBDE_ERR_INVALID, std::string("nvrtcCreateProgram: ") + nv.err_str(r));
  const char* opts[] = {"--gpu-architecture=sm_103a", "-std=c++17",
                        "-default-device", "-lineinfo"};
  r = nv.compile(prog, (int)(sizeof(opts) / sizeof(opts[0])), opts);
  if (r != NVRTC_SUCCESS) {
    size_t n = 0;
    nv.log_size(prog, &n);
    std::string log(n, '\0');
    if (n) nv.log(prog, &log[0]);
    nv.destroy(&prog);
    if (log.size() > 3000) log = log.substr(0, 3000) + "\n...";
    return fail(GBDE_ERR_INVALID, "model '" + label + "'" + (cb ? " with its callback" : "") +
                                      " does not compile for " + alg_type(alg, precision) +
                                      ":\n" + log);
  }
  size_t n = 0;
  nv.cubin_size(prog, &n);
  Compiled c;
  c.cubin.resize(n);
  nv.cubin(prog, c.cubin.data());
  nv.destroy(&prog);
  *out = &(g_compiled[key] = std::move(c));
  return GBDE_OK;
}

}  // namespace

namespace gbde {

bool rtc_model_info(int id, int32_t* n_state, int32_t* n_param) {
  std::lock_guard<std::mutex> lk(g_mu);
  const UserModelDef* m = find_model(id);
  if (!m) return false;
  if (n_state) *n_state = m->n;
  if (n_param) *n_param = m->np;
  return true;
}

bool rtc_model_has_noise(int id) {
  std::lock_guard<std::mutex> lk(g_mu);
  const UserModelDef* m = find_model(id);
  return m && !m->g_body.empty();
}

// Compile (if not cached) and load the kernels of (model, alg, precision).
// Called before any work is enqueued, so never inside a stream capture.
int rtc_prepare(int id, int alg, int precision, int callback, std::string* err) {
  std::lock_guard<std::mutex> lk(g_mu);
  Compiled* c = nullptr;
  int rc = compile_locked(id, alg, precision, callback, &c);
  if (rc != GBDE_OK) {
    if (err) *err = gbde_last_error(nullptr);
    return rc;
  }
  if (c->lib == nullptr) {
    cudaError_t e = cudaLibraryLoadData(&c->lib, c->cubin.data(), nullptr, nullptr, 0, nullptr,
                                        nullptr, 0);
    if (e == cudaSuccess) e = cudaLibraryGetKernel(&c->step, c->lib, "gbde_rtc_step");
    if (e == cudaSuccess) e = cudaLibraryGetKernel(&c->init, c->lib, "gbde_rtc_init_dt");
    if (e != cudaSuccess) {
      if (c->lib) cudaLibraryUnload(c->lib);
      c->lib = nullptr;
      if (err) *err = std::string("loading the compiled model failed: ") + cudaGetErrorString(e);
      return GBDE_ERR_CUDA;
    }
  }
  // load both kernels into the current device's context now (a library
  // loads lazily on first use, which must not happen inside a stream capture)
  cudaFuncAttributes fa;
  cudaError_t e = cudaFuncGetAttributes(&fa, (const void*)c->step);
  if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, (const void*)c->init);
  if (e != cudaSuccess) {
    if (err) *err = std::string("loading the compiled model failed: ") + cudaGetErrorString(e);
    return GBDE_ERR_CUDA;
  }
  return GBDE_OK;
}

// Launch a prepared user-model solve: the initial-dt pre-pass when
// cfg.dt_init is set, then the step kernel (plain or persistent geometry as
// launch_kernel).
cudaError_t launch_rtc(const LaunchCfg& cfg, const KArgs& a, cudaStream_t s) {
  cudaKernel_t step = nullptr, init = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_mu);
    auto it = g_compiled.find(std::make_tuple(cfg.model, cfg.alg, cfg.precision, cfg.callback));
    if (it == g_compiled.end() || it->second.lib == nullptr) return cudaErrorInvalidResourceHandle;
    step = it->second.step;
    init = it->second.init;
  }
  KArgs b = a;
  if (cfg.dt_init != nullptr) {
    const long long want = (a.N + 127) / 128, cap = 8LL * cfg.num_sms;
    const int g = (int)(want < cap ? (want > 0 ? want : 1) : cap);
    double* out = cfg.dt_init;
    void* args[] = {(void*)&a, (void*)&out};
    cudaError_t e = cudaLaunchKernel((const void*)init, dim3(g), dim3(128), args, 0, s);
    if (e != cudaSuccess) return e;
    b.dt_init = cfg.dt_init;
  }
  const int block = cfg.block > 0 ? cfg.block : 128;
  int grid;
  if (cfg.persistent) {
    int per_sm = cfg.ctas_per_sm;
    if (per_sm <= 0) {
      cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, (const void*)step,
                                                                    block, 0);
      if (e != cudaSuccess) return e;
      if (per_sm < 1) per_sm = 1;
    }
    grid = per_sm * cfg.num_sms;
    const long long need = (b.N + block - 1) / block;
    if (grid > need) grid = (int)(need > 0 ? need : 1);
  } else {
    const long long g = (b.N + block - 1) / block;
    grid = (int)(g > 0 ? g : 1);
  }
  void* args[] = {(void*)&b};
  return cudaLaunchKernel((const void*)step, dim3(grid), dim3(block), args, 0, s);
}

}  // namespace gbde

extern "C" {

static int register_model(const gbde_user_model* def, const char* g_body, int32_t* model_id) {
  if (!def || !model_id || !def->f_body)
    return fail(GBDE_ERR_INVALID, "def, def->f_body and model_id must be non-NULL");
  if (def->n_state < 1 || def->n_state > GBDE_USER_MAX_STATE)
    return fail(GBDE_ERR_INVALID, "user models have 1 to 8 states (one thread per trajectory)");
  if (def->n_param < 1 || def->n_param > GBDE_USER_MAX_PARAM)
    return fail(GBDE_ERR_INVALID, "user models have 1 to 32 parameters");
  UserModelDef m;
  m.name = def->name && def->name[0] ? def->name : "user_model";
  for (char& ch : m.name)
    if (!((ch >= 'a' && ch <= 'z') || (ch >= 'A' && ch <= 'Z') || (ch >= '0' && ch <= '9'))) ch = '_';
  m.f_body = def->f_body;
  m.jac_body = def->jac_body ? def->jac_body : "";
  m.g_body = g_body ? g_body : "";
  m.n = def->n_state;
  m.np = def->n_param;
  std::lock_guard<std::mutex> lk(g_mu);
  *model_id = GBDE_MODEL_USER_BASE + (int32_t)g_models.size();
  g_models.push_back(std::move(m));
  return GBDE_OK;
}

int gbde_model_register(const gbde_user_model* def, int32_t* model_id) {
  return register_model(def, nullptr, model_id);
}

int gbde_sde_model_register(const gbde_user_model* def, const char* g_body, int32_t* model_id) {
  if (!g_body || !g_body[0])
    return fail(GBDE_ERR_INVALID, "g_body (the diagonal noise) must be non-empty");
  return register_model(def, g_body, model_id);
}

int gbde_model_compile(int32_t model_id, int32_t alg, int32_t precision) {
  std::lock_guard<std::mutex> lk(g_mu);
  Compiled* c = nullptr;
  return compile_locked(model_id, alg, precision, 0, &c);
}

static int push_callback(CallbackDef&& c, int32_t* callback_id) {
  std::lock_guard<std::mutex> lk(g_mu);
  for (int id : c.members)
    if (!find_callback(id))
      return fail(GBDE_ERR_INVALID, "unknown callback id " + std::to_string(id) + " in the set");
  g_callbacks.push_back(std::move(c));
  *callback_id = (int32_t)g_callbacks.size();
  return GBDE_OK;
}

static int leaf_callback(const gbde_callback* def, int kind, int len, int32_t* callback_id) {
  if (!def || !callback_id || !def->condition)
    return fail(GBDE_ERR_INVALID, "def, def->condition and callback_id must be non-NULL");
  CallbackDef c;
  c.kind = kind;
  c.len = len;
  if (def->save_positions & ~(GBDE_SAVE_BEFORE | GBDE_SAVE_AFTER))
    return fail(GBDE_ERR_INVALID, "save_positions takes GBDE_SAVE_BEFORE | GBDE_SAVE_AFTER bits");
  c.condition = def->condition;
  c.affect = def->affect ? def->affect : "";
  c.has_affect = def->affect != nullptr || def->terminate;
  c.save = def->save_positions;
  if (def->terminate) c.affect += "\nterminate = true;";
  return push_callback(std::move(c), callback_id);
}

int gbde_callback_register(const gbde_callback* def, int32_t* callback_id) {
  if (def && def->kind != GBDE_CB_CONTINUOUS && def->kind != GBDE_CB_DISCRETE)
    return fail(GBDE_ERR_INVALID, "kind must be GBDE_CB_CONTINUOUS or GBDE_CB_DISCRETE");
  return leaf_callback(def, def ? def->kind : 0, 1, callback_id);
}

int gbde_vector_callback_register(const gbde_callback* def, int32_t len, int32_t* callback_id) {
  if (len < 1 || len > GBDE_MAX_CB_CONDITIONS)
    return fail(GBDE_ERR_INVALID, "len must be in [1, " + std::to_string(GBDE_MAX_CB_CONDITIONS) + "]");
  if (def && def->kind != GBDE_CB_VECTOR)
    return fail(GBDE_ERR_INVALID, "kind must be GBDE_CB_VECTOR");
  return leaf_callback(def, GBDE_CB_VECTOR, len, callback_id);
}

int gbde_callback_set_register(const int32_t* ids, int32_t n, int32_t* set_id) {
  if (!ids || !set_id || n < 1)
    return fail(GBDE_ERR_INVALID, "ids and set_id must be non-NULL and n >= 1");
  CallbackDef c;
  c.members.assign(ids, ids + n);
  return push_callback(std::move(c), set_id);
}

int gbde_callback_compile(int32_t model, int32_t alg, int32_t precision, int32_t callback_id) {
  std::lock_guard<std::mutex> lk(g_mu);
  Compiled* c = nullptr;
  return compile_locked(model, alg, precision, callback_id, &c);
}

}  // extern "C"
