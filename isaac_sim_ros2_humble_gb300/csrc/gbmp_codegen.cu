// gbmp_codegen.cu -- runtime code generation of robot-specific kernels.
//
// Replaces the reference's genForwardKinematicsKernelCode / get_step / interpolate
// generators (KernelGenerator.h:222-522) and its NVRTC loader KernelFunction::create
// (NvrtcUtil.h:58-148):
//   * the generator writes one CUDA C++ translation unit per robot in which every joint
//     pose, axis, parent index, joint type and sphere offset is a literal (bit patterns,
//     so nothing is lost in printing), the link chain is unrolled and each thread owns
//     one joint state in registers;
//   * the source is compiled by NVRTC for the device's own architecture (sm_103a on
//     GB300) straight to a cubin and loaded with cudaLibraryLoadData;
//   * cubins are cached in process by a 64-bit FNV-1a hash of (source, architecture,
//     NVRTC version) and, when GBMP_CODEGEN_CACHE names a directory, on disk under that
//     hash (the reference keys its disk cache by kernel name only, so two robots in one
//     working directory overwrite each other).
// The arithmetic of the generated FK is the table-driven kernels' (joint_local,
// mul_elem, xform_point in gbmp_device.cuh) written out operation by operation with
// the same rounding intrinsics, so both give bit-identical poses and sphere centres.
// NVRTC is opened with dlopen, so libgbmp loads and runs without it; only robots
// created with GBMP_ROBOT_CODEGEN need it.
#include <dlfcn.h>
#include <nvrtc.h>

#include <chrono>
#include <climits>
#include <cstring>
#include <fstream>
#include <map>
#include <memory>
#include <sstream>

#include "gbmp_internal.h"

namespace gbmp {

// ---------------------------------------------------------------------------------
// NVRTC entry points (dlopen).
// ---------------------------------------------------------------------------------
struct Nvrtc {
    void *h = nullptr;
    nvrtcResult (*create)(nvrtcProgram *, const char *, const char *, int, const char *const *,
                          const char *const *) = nullptr;
    nvrtcResult (*compile)(nvrtcProgram, int, const char *const *) = nullptr;
    nvrtcResult (*log_size)(nvrtcProgram, size_t *) = nullptr;
    nvrtcResult (*log)(nvrtcProgram, char *) = nullptr;
    nvrtcResult (*cubin_size)(nvrtcProgram, size_t *) = nullptr;
    nvrtcResult (*cubin)(nvrtcProgram, char *) = nullptr;
    nvrtcResult (*destroy)(nvrtcProgram *) = nullptr;
    nvrtcResult (*version)(int *, int *) = nullptr;
    const char *(*err)(nvrtcResult) = nullptr;
    std::string why;
};

static Nvrtc &nvrtc() {
    static Nvrtc api;
    static std::once_flag once;
    std::call_once(once, [] {
        const char *names[] = {"libnvrtc.so.13", "libnvrtc.so", "/usr/local/cuda/lib64/libnvrtc.so"};
        for (const char *n : names)
            if ((api.h = dlopen(n, RTLD_NOW | RTLD_LOCAL))) break;
        if (!api.h) {
            api.why = "libnvrtc could not be opened";
            return;
        }
        bool ok = true;
        auto sym = [&](auto &fn, const char *name) {
            fn = reinterpret_cast<std::remove_reference_t<decltype(fn)>>(dlsym(api.h, name));
            ok &= fn != nullptr;
        };
        sym(api.create, "nvrtcCreateProgram");
        sym(api.compile, "nvrtcCompileProgram");
        sym(api.log_size, "nvrtcGetProgramLogSize");
        sym(api.log, "nvrtcGetProgramLog");
        sym(api.cubin_size, "nvrtcGetCUBINSize");
        sym(api.cubin, "nvrtcGetCUBIN");
        sym(api.destroy, "nvrtcDestroyProgram");
        sym(api.version, "nvrtcVersion");
        sym(api.err, "nvrtcGetErrorString");
        if (!ok) {
            api.why = "libnvrtc lacks an expected entry point";
            dlclose(api.h);
            api.h = nullptr;
        }
    });
    return api;
}

// ---------------------------------------------------------------------------------
// Source generation.
// ---------------------------------------------------------------------------------
namespace {

std::string flit(float v) {
    unsigned u;
    memcpy(&u, &v, 4);
    char b[40];
    snprintf(b, sizeof b, "__int_as_float(0x%08xu)", u);
    return b;
}

std::string var(int link, int e) { return "t" + std::to_string(link) + "_" + std::to_string(e); }

struct Src {
    std::ostringstream o;
    template <typename... A>
    void line(const char *fmt, A... a) {
        if constexpr (sizeof...(A) == 0) {
            o << fmt << '\n';
        } else {
            char b[1024];
            snprintf(b, sizeof b, fmt, a...);
            o << b << '\n';
        }
    }
};

// Link i's pose t<i>_0..11 from its parent's and its joint's local transform
// (joint_local + mul_elem).
void emit_link(Src &s, const gbmp_robot_s *r, int i, const float *jl, const float *axn, const float *axr) {
    const int ty = r->type[i], p = r->parent[i];
    const float *P = jl + 12 * i;
    if (ty != 1 && ty != 2 && ty != 5) {
        for (int e = 0; e < 12; ++e)
            s.line("    const float %s = %s;", var(i, e).c_str(), (e % 5 == 0) ? "1.f" : "0.f");
        return;
    }
    s.line("    float m%d[12];", i);
    if (ty == 1) {
        const float *n = axn + 4 * i;
        s.line("    {");
        s.line("      float sn, cs;");
        s.line("      sincosf(q[%d], &sn, &cs);", i);
        const std::string nx = flit(n[0]), ny = flit(n[1]), nz = flit(n[2]), va = flit(n[3]);
        s.line("      const float nx = %s, ny = %s, nz = %s, va = %s;", nx.c_str(), ny.c_str(), nz.c_str(), va.c_str());
        s.line("      const float oc = __fadd_rn(1.f, -cs), iv = __fadd_rn(1.f, -va);");
        s.line("      float R[9];");
        s.line("      R[0] = __fadd_rn(__fmul_rn(__fmaf_rn(__fmul_rn(nx, nx), oc, cs), va), iv);");
        s.line("      R[1] = __fmul_rn(__fmaf_rn(__fmul_rn(nx, ny), oc, -__fmul_rn(nz, sn)), va);");
        s.line("      R[2] = __fmul_rn(__fmaf_rn(__fmul_rn(nx, nz), oc, __fmul_rn(ny, sn)), va);");
        s.line("      R[3] = __fmul_rn(__fmaf_rn(__fmul_rn(ny, nx), oc, __fmul_rn(nz, sn)), va);");
        s.line("      R[4] = __fadd_rn(__fmul_rn(__fmaf_rn(__fmul_rn(ny, ny), oc, cs), va), iv);");
        s.line("      R[5] = __fmul_rn(__fmaf_rn(__fmul_rn(ny, nz), oc, -__fmul_rn(nx, sn)), va);");
        s.line("      R[6] = __fmul_rn(__fmaf_rn(__fmul_rn(nz, nx), oc, -__fmul_rn(ny, sn)), va);");
        s.line("      R[7] = __fmul_rn(__fmaf_rn(__fmul_rn(nz, ny), oc, __fmul_rn(nx, sn)), va);");
        s.line("      R[8] = __fadd_rn(__fmul_rn(__fmaf_rn(__fmul_rn(nz, nz), oc, cs), va), iv);");
        for (int rr = 0; rr < 3; ++rr) {
            const std::string a = flit(P[4 * rr]), b = flit(P[4 * rr + 1]), c = flit(P[4 * rr + 2]),
                              d = flit(P[4 * rr + 3]);
            for (int cc = 0; cc < 3; ++cc)
                s.line("      m%d[%d] = __fmaf_rn(%s, R[%d], __fmaf_rn(%s, R[%d], __fmul_rn(%s, R[%d])));", i,
                       4 * rr + cc, c.c_str(), 6 + cc, b.c_str(), 3 + cc, a.c_str(), cc);
            s.line("      m%d[%d] = __fadd_rn(__fmaf_rn(%s, 0.f, __fmaf_rn(%s, 0.f, __fmul_rn(%s, 0.f))), %s);", i,
                   4 * rr + 3, c.c_str(), b.c_str(), a.c_str(), d.c_str());
        }
        s.line("    }");
    } else if (ty == 2) {
        const float *a = axr + 4 * i;
        s.line("    {");
        s.line("      const float tx = __fmul_rn(%s, q[%d]), ty = __fmul_rn(%s, q[%d]), tz = __fmul_rn(%s, q[%d]);",
               flit(a[0]).c_str(), i, flit(a[1]).c_str(), i, flit(a[2]).c_str(), i);
        for (int rr = 0; rr < 3; ++rr) {
            const std::string A = flit(P[4 * rr]), B = flit(P[4 * rr + 1]), C = flit(P[4 * rr + 2]),
                              D = flit(P[4 * rr + 3]);
            for (int cc = 0; cc < 3; ++cc)
                s.line("      m%d[%d] = __fmaf_rn(%s, %s, __fmaf_rn(%s, %s, __fmul_rn(%s, %s)));", i, 4 * rr + cc,
                       C.c_str(), cc == 2 ? "1.f" : "0.f", B.c_str(), cc == 1 ? "1.f" : "0.f", A.c_str(),
                       cc == 0 ? "1.f" : "0.f");
            s.line("      m%d[%d] = __fadd_rn(__fmaf_rn(%s, tz, __fmaf_rn(%s, ty, __fmul_rn(%s, tx))), %s);", i,
                   4 * rr + 3, C.c_str(), B.c_str(), A.c_str(), D.c_str());
        }
        s.line("    }");
    } else {
        for (int e = 0; e < 12; ++e) s.line("    m%d[%d] = %s;", i, e, flit(P[e]).c_str());
    }
    for (int rr = 0; rr < 3; ++rr)
        for (int cc = 0; cc < 4; ++cc) {
            const std::string a0 = var(p, 4 * rr), a1 = var(p, 4 * rr + 1), a2 = var(p, 4 * rr + 2);
            if (cc < 3)
                s.line("    const float %s = __fmaf_rn(%s, m%d[%d], __fmaf_rn(%s, m%d[%d], __fmul_rn(%s, m%d[%d])));",
                       var(i, 4 * rr + cc).c_str(), a2.c_str(), i, 8 + cc, a1.c_str(), i, 4 + cc, a0.c_str(), i, cc);
            else
                s.line("    const float %s = __fadd_rn(__fmaf_rn(%s, m%d[11], __fmaf_rn(%s, m%d[7], __fmul_rn(%s, "
                       "m%d[3]))), %s);",
                       var(i, 4 * rr + 3).c_str(), a2.c_str(), i, a1.c_str(), i, a0.c_str(), i,
                       var(p, 4 * rr + 3).c_str());
        }
}

}  // namespace

std::string codegen_source(const gbmp_robot_s *r) {
    const int L = r->L, S = r->S;
    // the values uploaded for the table-driven kernels: jl (3x4 rows of each joint
    // pose), axn (normalised axis + valid flag), axr (raw axis)
    const std::vector<float> &jl = r->h_jl, &axn = r->h_axn, &axr = r->h_axr;
    Src s;
    s.line("// Generated by libgbmp for one robot: %d links, %d spheres.  Thread per joint state.", L, S);
    s.line("#define GBMP_L %d", L);
    s.line("#define GBMP_S %d", S);
    s.line("");
    s.line("extern \"C\" __global__ void __launch_bounds__(128) gbmp_gen_fk(const float *__restrict__ qall, long long n,");
    s.line("                                                              float *__restrict__ poses, float *__restrict__ centers) {");
    s.line("  const long long st = blockIdx.x * (long long)blockDim.x + threadIdx.x;");
    s.line("  if (st >= n) return;");
    s.line("  float q[GBMP_L];");
    s.line("#pragma unroll");
    s.line("  for (int j = 0; j < GBMP_L; ++j) q[j] = qall[st * GBMP_L + j];");
    for (int e = 0; e < 12; ++e) s.line("  const float %s = %s;", var(0, e).c_str(), (e % 5 == 0) ? "1.f" : "0.f");
    for (int i = 1; i < L; ++i) {
        s.line("  // link %d: type %d, parent %d", i, r->type[i], r->parent[i]);
        emit_link(s, r, i, jl.data(), axn.data(), axr.data());
    }
    s.line("  if (poses) {");
    s.line("    float *P = poses + st * (GBMP_L * 16);");
    for (int i = 0; i < L; ++i) {
        for (int e = 0; e < 12; ++e) s.line("    P[%d] = %s;", 16 * i + e, var(i, e).c_str());
        s.line("    P[%d] = 0.f; P[%d] = 0.f; P[%d] = 0.f; P[%d] = 1.f;", 16 * i + 12, 16 * i + 13, 16 * i + 14,
               16 * i + 15);
    }
    s.line("  }");
    s.line("  if (centers) {");
    s.line("    float *C = centers + st * (GBMP_S * 3);");
    for (int k = 0; k < S; ++k) {
        const int l = r->slink[k];
        const std::string x = flit(r->sph_pos[3 * k]), y = flit(r->sph_pos[3 * k + 1]), z = flit(r->sph_pos[3 * k + 2]);
        for (int c = 0; c < 3; ++c)
            s.line("    C[%d] = __fadd_rn(__fmaf_rn(%s, %s, __fmaf_rn(%s, %s, __fmul_rn(%s, %s))), %s);", 3 * k + c,
                   var(l, 4 * c + 2).c_str(), z.c_str(), var(l, 4 * c + 1).c_str(), y.c_str(),
                   var(l, 4 * c).c_str(), x.c_str(), var(l, 4 * c + 3).c_str());
    }
    s.line("  }");
    s.line("}");
    s.line("");
    // Edge set-up (KernelGenerator.h:408-465 step + direction), k_edge_setup with L fixed.
    s.line("extern \"C\" __global__ void __launch_bounds__(256) gbmp_gen_edge_setup(");
    s.line("    const float *__restrict__ from, const float *__restrict__ to, long long E, float res, int rule,");
    s.line("    int *__restrict__ nsteps, float *__restrict__ dir, int *__restrict__ hist,");
    s.line("    float *__restrict__ length_out, int *__restrict__ nsteps_out) {");
    s.line("  const long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x;");
    s.line("  if (k >= E) return;");
    s.line("  const float *f = from + k * GBMP_L, *t = to + k * GBMP_L;");
    s.line("  float d2 = 0.f, dinf = 0.f;");
    s.line("#pragma unroll");
    s.line("  for (int j = 0; j < GBMP_L; ++j) {");
    s.line("    const float d = __fadd_rn(f[j], -t[j]);");
    s.line("    d2 = __fmaf_rn(d, d, d2);");
    s.line("    dinf = fmaxf(dinf, fabsf(d));");
    s.line("  }");
    s.line("  const float len = __fsqrt_rn(d2);");
    s.line("  const float metric = rule == %d ? dinf : len;", GBMP_STEP_LINF);
    s.line("  const float ratio = __fdiv_rn(metric, res);");
    s.line("  const int n = ratio < %d.0f ? (int)ratio + 1 : %d;", kMaxEdgeStates, kMaxEdgeStates + 1);
    s.line("  const float fn = (float)n;");
    s.line("#pragma unroll");
    s.line("  for (int j = 0; j < GBMP_L; ++j) dir[k * GBMP_L + j] = __fdiv_rn(__fadd_rn(t[j], -f[j]), fn);");
    s.line("  nsteps[k] = n;");
    s.line("  const int b = n >> 4;");
    s.line("  atomicAdd(hist + (%d - (b < %d ? b : %d)), 1);", kEdgeBuckets - 1, kEdgeBuckets - 1, kEdgeBuckets - 1);
    s.line("  if (length_out) length_out[k] = len;");
    s.line("  if (nsteps_out) nsteps_out[k] = n;");
    s.line("}");
    return s.o.str();
}

// ---------------------------------------------------------------------------------
// Compilation, caching, loading.
// ---------------------------------------------------------------------------------
static uint64_t fnv1a(const std::string &s, uint64_t h = 1469598103934665603ULL) {
    for (unsigned char c : s) {
        h ^= c;
        h *= 1099511628211ULL;
    }
    return h;
}

static std::mutex g_cache_mu;
static std::map<uint64_t, std::string> g_cubins;

static gbmp_status compile_cubin(const std::string &src, const std::string &arch, std::string *cubin,
                                 double *ms) {
    Nvrtc &api = nvrtc();
    if (!api.h) {
        set_error("runtime code generation unavailable: %s", api.why.c_str());
        return GBMP_ERR_CODEGEN;
    }
    const auto t0 = std::chrono::steady_clock::now();
    nvrtcProgram prog = nullptr;
    nvrtcResult e = api.create(&prog, src.c_str(), "gbmp_robot.cu", 0, nullptr, nullptr);
    if (e != NVRTC_SUCCESS) {
        set_error("nvrtcCreateProgram: %s", api.err(e));
        return GBMP_ERR_CODEGEN;
    }
    const std::string a = "--gpu-architecture=" + arch;
    const char *opts[] = {a.c_str(), "--std=c++17", "-lineinfo"};
    e = api.compile(prog, 3, opts);
    if (e != NVRTC_SUCCESS) {
        size_t n = 0;
        api.log_size(prog, &n);
        std::string log(n, '\0');
        if (n) api.log(prog, &log[0]);
        api.destroy(&prog);
        set_error("NVRTC compilation for %s failed: %s\n%s", arch.c_str(), api.err(e), log.c_str());
        return GBMP_ERR_CODEGEN;
    }
    size_t n = 0;
    e = api.cubin_size(prog, &n);
    if (e == NVRTC_SUCCESS && n) {
        cubin->resize(n);
        e = api.cubin(prog, &(*cubin)[0]);
    }
    api.destroy(&prog);
    if (e != NVRTC_SUCCESS || !n) {
        set_error("NVRTC gave no cubin for %s", arch.c_str());
        return GBMP_ERR_CODEGEN;
    }
    *ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    return GBMP_OK;
}

gbmp_status codegen_build(gbmp_robot_s *r) {
    int major = 0, minor = 0;
    GBMP_CUDA(cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, r->device));
    GBMP_CUDA(cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, r->device));
    char arch[32];
    snprintf(arch, sizeof arch, major >= 9 ? "sm_%d%da" : "sm_%d%d", major, minor);
    auto cg = std::make_unique<Codegen>();
    cg->source = codegen_source(r);
    int vmaj = 0, vmin = 0;
    if (nvrtc().h) nvrtc().version(&vmaj, &vmin);
    cg->arch = arch;
    cg->hash = fnv1a(cg->source + "|" + arch + "|" + std::to_string(vmaj) + "." + std::to_string(vmin));
    char hex[17];
    snprintf(hex, sizeof hex, "%016llx", (unsigned long long)cg->hash);
    std::string cubin;
    {
        std::lock_guard<std::mutex> lock(g_cache_mu);
        auto it = g_cubins.find(cg->hash);
        if (it != g_cubins.end()) {
            cubin = it->second;
            cg->cache = 1;
        }
    }
    const char *dir = getenv("GBMP_CODEGEN_CACHE");
    const std::string path = dir && *dir ? std::string(dir) + "/gbmp_" + hex + ".cubin" : std::string();
    if (cubin.empty() && !path.empty()) {
        std::ifstream in(path, std::ios::binary);
        if (in) {
            std::ostringstream ss;
            ss << in.rdbuf();
            cubin = ss.str();
            if (!cubin.empty()) cg->cache = 2;
        }
    }
    if (cubin.empty()) {
        gbmp_status st = compile_cubin(cg->source, arch, &cubin, &cg->compile_ms);
        if (st) return st;
        if (!path.empty()) {
            const std::string tmp = path + ".tmp" + std::to_string((unsigned long long)(uintptr_t)r);
            std::ofstream out(tmp, std::ios::binary);
            out.write(cubin.data(), (std::streamsize)cubin.size());
            out.close();
            if (!out || rename(tmp.c_str(), path.c_str()) != 0) remove(tmp.c_str());
        }
    }
    {
        std::lock_guard<std::mutex> lock(g_cache_mu);
        g_cubins.emplace(cg->hash, cubin);
    }
    cudaError_t e = cudaLibraryLoadData(&cg->lib, cubin.data(), nullptr, nullptr, 0, nullptr, nullptr, 0);
    if (e == cudaSuccess) e = cudaLibraryGetKernel(&cg->fk, cg->lib, "gbmp_gen_fk");
    if (e == cudaSuccess) e = cudaLibraryGetKernel(&cg->edge_setup, cg->lib, "gbmp_gen_edge_setup");
    if (e != cudaSuccess) {
        if (cg->lib) cudaLibraryUnload(cg->lib);
        cg->lib = nullptr;
        set_error("loading the generated kernels failed: %s", cudaGetErrorString(e));
        return GBMP_ERR_CODEGEN;
    }
    r->cg = cg.release();
    return GBMP_OK;
}

void codegen_free(Codegen *cg) {
    if (!cg) return;
    if (cg->lib) cudaLibraryUnload(cg->lib);
    delete cg;
}

gbmp_status codegen_fk(const gbmp_robot_s *r, const float *q, long long n, float *poses, float *centers,
                       cudaStream_t s) {
    const int tb = 128;
    const unsigned blocks = (unsigned)((n + tb - 1) / tb);
    void *args[] = {(void *)&q, (void *)&n, (void *)&poses, (void *)&centers};
    ProfScope ps(GBMP_PROF_FK, s);
    GBMP_CUDA(cudaLaunchKernel((const void *)r->cg->fk, dim3(blocks), dim3(tb), args, 0, s));
    return GBMP_OK;
}

gbmp_status codegen_edge_setup(const gbmp_robot_s *r, const float *from, const float *to, long long E, float res,
                               int rule, int *nsteps, float *dir, int *hist, float *length_out, int *nsteps_out,
                               cudaStream_t s) {
    const int tb = 256;
    const unsigned blocks = (unsigned)((E + tb - 1) / tb);
    void *args[] = {(void *)&from,  (void *)&to,   (void *)&E,    (void *)&res,
                    (void *)&rule,  (void *)&nsteps, (void *)&dir, (void *)&hist,
                    (void *)&length_out, (void *)&nsteps_out};
    ProfScope ps(GBMP_PROF_OTHER, s);
    GBMP_CUDA(cudaLaunchKernel((const void *)r->cg->edge_setup, dim3(blocks), dim3(tb), args, 0, s));
    return GBMP_OK;
}

}  // namespace gbmp

using namespace gbmp;

extern "C" {

gbmp_status gbmp_robot_codegen_info(gbmp_robot r, char *source, int64_t capacity, int64_t *source_len,
                                    uint64_t *hash, int32_t *cache, double *compile_ms) {
    GBMP_CHECK_ARG(r, "robot is NULL");
    if (!r->cg) {
        set_error("robot was created without GBMP_ROBOT_CODEGEN");
        return GBMP_ERR_UNSUPPORTED;
    }
    const std::string &src = r->cg->source;
    if (source_len) *source_len = (int64_t)src.size() + 1;
    if (source) {
        GBMP_CHECK_ARG(capacity >= (int64_t)src.size() + 1, "source needs %lld bytes, capacity %lld",
                       (long long)src.size() + 1, (long long)capacity);
        memcpy(source, src.c_str(), src.size() + 1);
    }
    if (hash) *hash = r->cg->hash;
    if (cache) *cache = r->cg->cache;
    if (compile_ms) *compile_ms = r->cg->compile_ms;
    return GBMP_OK;
}

}  // extern "C"
