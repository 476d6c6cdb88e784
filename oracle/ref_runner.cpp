// Runs the reference's own CUDA kernels (PTX compiled from CosmosCuda.cuh by
// oracle/ref_build.py) on the GPU -- TEST INFRASTRUCTURE, the GPU half of the
// oracle.  Used by tests/golden/make_golden.py to produce golden fixtures and by
// bench.py to time the reference's step on the same GPU.
//
// The host side restates the single-GPU sequence of Universe<K>
// (CosmosCuda.cuh):
//   constructor  :969-1029  buffers, numBlocks = SMs * ceil(maxThreadsPerSM / 768),
//                           k_generateFilterLattice, k_generateMassAssignmentKernel,
//                           cufftPlan2d(N, N, C2C), forward FFT of both,
//                           CIC: k_applyPhaseShift(-0.5, -0.5)
//   step         :1240-1263 k_clearAccumulator, k_scatterMassOnAccumulator,
//                           k_copyAccumulatorIntoLattice, (CIC) k_getRealComponentOfLattice
//                :1266      cufftExecC2C forward
//                :1286-1287 k_multElementwiseLatticeFilter, k_divElementwiseLatticeFilter
//                :1291      cufftExecC2C inverse
//                :1297-1299 k_shiftLattice, k_calcGradientLattice, k_forceMultiSampling
//   render       :1249-1256 k_getRealComponentOfLattice, k_calcBlurConvolution,
//                           k_resetMinMax, k_calcMinMax, k_smoothMinMax,
//                           k_scaleWithMinMax (ref_render, on a given density;
//                           the running extremes start with k_initSmoothMinMax)
// Kernels are looked up by their demangled names in the loaded module.
#include <cuda.h>
#include <cuda_runtime.h>
#include <cufft.h>
#include <cxxabi.h>

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

namespace {

thread_local std::string g_err;

int fail(const std::string& m) {
    g_err = m;
    return -1;
}

#define RR_CU(call)                                                                         \
    do {                                                                                    \
        CUresult r_ = (call);                                                               \
        if (r_ != CUDA_SUCCESS) {                                                           \
            const char* s_ = nullptr;                                                       \
            cuGetErrorString(r_, &s_);                                                      \
            return fail(std::string(#call) + ": " + (s_ ? s_ : "?"));                       \
        }                                                                                   \
    } while (0)
#define RR_RT(call)                                                                         \
    do {                                                                                    \
        cudaError_t e_ = (call);                                                            \
        if (e_ != cudaSuccess) return fail(std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)
#define RR_FFT(call)                                                                        \
    do {                                                                                    \
        cufftResult f_ = (call);                                                            \
        if (f_ != CUFFT_SUCCESS) return fail(std::string(#call) + ": cufft error " + std::to_string(int(f_))); \
    } while (0)

const char* kKernels[] = {"k_generateFilterLattice",        "k_generateMassAssignmentKernel",
                          "k_applyPhaseShift",              "k_clearAccumulator",
                          "k_scatterMassOnAccumulator",     "k_copyAccumulatorIntoLattice",
                          "k_getRealComponentOfLattice",    "k_multElementwiseLatticeFilter",
                          "k_divElementwiseLatticeFilter",  "k_shiftLattice",
                          "k_calcGradientLattice",          "k_forceMultiSampling",
                          "k_calcBlurConvolution",          "k_resetMinMax",
                          "k_calcMinMax",                   "k_initSmoothMinMax",
                          "k_smoothMinMax",                 "k_scaleWithMinMax"};

struct Ref {
    int N = 0, P = 0;
    bool accuracy = false;  // CIC
    CUmodule mod = nullptr;
    std::map<std::string, CUfunction> fn;
    cudaStream_t st = nullptr;
    cufftHandle plan = 0;
    int numBlocks = 0;
    float2 *lattice = nullptr, *filter = nullptr, *deconv = nullptr, *forceXY = nullptr;
    float *acc = nullptr, *shifted = nullptr, *localForce = nullptr;
    float *render1 = nullptr, *render2 = nullptr;  // renderOutput_d, renderOutput2_d
    float *x = nullptr, *y = nullptr, *xo = nullptr, *yo = nullptr, *m = nullptr;
};

int launch_shape(Ref* r, const char* name, dim3 grid, dim3 block, unsigned smem, std::vector<void*> args) {
    auto it = r->fn.find(name);
    if (it == r->fn.end()) return fail(std::string("kernel not found: ") + name);
    RR_CU(cuLaunchKernel(it->second, grid.x, grid.y, grid.z, block.x, block.y, block.z, smem,
                         reinterpret_cast<CUstream>(r->st), args.data(), nullptr));
    return 0;
}

// The reference's usual shape: numBlocks x THREADS (768).
int launch(Ref* r, const char* name, std::vector<void*> args) {
    return launch_shape(r, name, dim3(r->numBlocks), dim3(768), 0, std::move(args));
}

int load_module(Ref* r, const char* ptx_path) {
    std::ifstream f(ptx_path, std::ios::binary);
    if (!f) return fail(std::string("cannot open ") + ptx_path);
    std::stringstream ss;
    ss << f.rdbuf();
    const std::string ptx = ss.str();
    RR_CU(cuModuleLoadData(&r->mod, ptx.c_str()));
    unsigned int count = 0;
    RR_CU(cuModuleGetFunctionCount(&count, r->mod));
    std::vector<CUfunction> fs(count);
    RR_CU(cuModuleEnumerateFunctions(fs.data(), count, r->mod));
    for (CUfunction f1 : fs) {
        const char* mangled = nullptr;
        RR_CU(cuFuncGetName(&mangled, f1));
        int status = 0;
        char* dem = abi::__cxa_demangle(mangled, nullptr, nullptr, &status);
        const std::string d = (status == 0 && dem) ? dem : mangled;
        std::free(dem);
        for (const char* k : kKernels) {  // templates end in '<', plain kernels in '('
            const std::string key = std::string("Kernels::") + k;
            const size_t at = d.find(key);
            if (at != std::string::npos && at + key.size() < d.size() &&
                (d[at + key.size()] == '<' || d[at + key.size()] == '('))
                r->fn[k] = f1;
        }
    }
    for (const char* k : kKernels)
        if (!r->fn.count(k)) return fail(std::string("reference kernel missing from module: ") + k);
    return 0;
}

int create(Ref* r, const char* ptx_path, int N, int cic, int P) {
    r->N = N;
    r->P = P;
    r->accuracy = cic != 0;
    RR_RT(cudaFree(nullptr));  // primary context
    RR_CU(cuInit(0));
    if (load_module(r, ptx_path)) return -1;
    RR_RT(cudaStreamCreate(&r->st));
    int dev = 0;
    RR_RT(cudaGetDevice(&dev));
    cudaDeviceProp prop;
    RR_RT(cudaGetDeviceProperties(&prop, dev));
    r->numBlocks = prop.multiProcessorCount * ((prop.maxThreadsPerMultiProcessor + 768 - 1) / 768);
    const size_t NN = size_t(N) * N;
    RR_RT(cudaMalloc(&r->lattice, NN * sizeof(float2)));
    RR_RT(cudaMalloc(&r->filter, NN * sizeof(float2)));
    RR_RT(cudaMalloc(&r->deconv, NN * sizeof(float2)));
    RR_RT(cudaMalloc(&r->forceXY, NN * sizeof(float2)));
    RR_RT(cudaMalloc(&r->acc, NN * sizeof(float)));
    RR_RT(cudaMalloc(&r->shifted, NN * sizeof(float)));
    RR_RT(cudaMalloc(&r->localForce, NN * sizeof(float)));
    RR_RT(cudaMalloc(&r->render1, NN * sizeof(float)));
    RR_RT(cudaMalloc(&r->render2, NN * sizeof(float)));
    // the reference's blur grid covers no tile when N < 1024; keep that frame defined
    RR_RT(cudaMemsetAsync(r->render2, 0, NN * sizeof(float), r->st));
    if (launch_shape(r, "k_initSmoothMinMax", dim3(1), dim3(1), 0, {})) return -1;
    // blur weights into the module's __constant__ table, as the constructor
    // does (:954-966, :981): 1/(r+1) for r < BLUR_HALF_R, BLUR_R = 3
    {
        CUdeviceptr kern = 0;
        size_t bytes = 0;
        RR_CU(cuModuleGetGlobal(&kern, &bytes, r->mod, "_ZN7Kernels16renderBlurKern_cE"));
        float w[9];
        for (int iy = -1; iy <= 1; ++iy)
            for (int ix = -1; ix <= 1; ++ix) {
                const double rr = std::sqrt(double(ix * ix + iy * iy));
                w[(ix + 1) + (iy + 1) * 3] = rr < 1 ? float(1.0 / (rr + 1.0)) : 0.0f;
            }
        if (bytes != sizeof(w)) return fail("renderBlurKern_c has an unexpected size");
        RR_CU(cuMemcpyHtoD(kern, w, sizeof(w)));
    }
    for (float** p : {&r->x, &r->y, &r->xo, &r->yo, &r->m}) RR_RT(cudaMalloc(p, size_t(P > 0 ? P : 1) * sizeof(float)));
    RR_RT(cudaMemsetAsync(r->acc, 0, NN * sizeof(float), r->st));
    RR_RT(cudaMemsetAsync(r->lattice, 0, NN * sizeof(float2), r->st));
    RR_RT(cudaMemsetAsync(r->shifted, 0, NN * sizeof(float), r->st));
    RR_RT(cudaMemsetAsync(r->forceXY, 0, NN * sizeof(float2), r->st));
    bool acc = r->accuracy;
    if (launch(r, "k_generateFilterLattice", {&r->filter, &acc})) return -1;
    if (launch(r, "k_generateMassAssignmentKernel", {&r->deconv, &acc})) return -1;
    RR_FFT(cufftPlan2d(&r->plan, N, N, CUFFT_C2C));
    RR_FFT(cufftSetStream(r->plan, r->st));
    RR_FFT(cufftExecC2C(r->plan, reinterpret_cast<cufftComplex*>(r->filter), reinterpret_cast<cufftComplex*>(r->filter),
                        CUFFT_FORWARD));
    RR_FFT(cufftExecC2C(r->plan, reinterpret_cast<cufftComplex*>(r->deconv), reinterpret_cast<cufftComplex*>(r->deconv),
                        CUFFT_FORWARD));
    if (acc) {
        float fx = -0.5f, fy = -0.5f;
        if (launch(r, "k_applyPhaseShift", {&r->deconv, &fx, &fy})) return -1;
    }
    RR_RT(cudaStreamSynchronize(r->st));
    return 0;
}

int step_once(Ref* r) {
    bool acc = r->accuracy;
    int P = r->P;
    if (launch(r, "k_clearAccumulator", {&r->acc})) return -1;
    if (launch(r, "k_scatterMassOnAccumulator", {&r->acc, &r->x, &r->y, &r->m, &P, &acc})) return -1;
    if (launch(r, "k_copyAccumulatorIntoLattice", {&r->acc, &r->lattice})) return -1;
    if (acc && launch(r, "k_getRealComponentOfLattice", {&r->lattice, &r->localForce})) return -1;
    RR_FFT(cufftExecC2C(r->plan, reinterpret_cast<cufftComplex*>(r->lattice),
                        reinterpret_cast<cufftComplex*>(r->lattice), CUFFT_FORWARD));
    if (launch(r, "k_multElementwiseLatticeFilter", {&r->lattice, &r->filter})) return -1;
    if (launch(r, "k_divElementwiseLatticeFilter", {&r->lattice, &r->deconv})) return -1;
    RR_FFT(cufftExecC2C(r->plan, reinterpret_cast<cufftComplex*>(r->lattice),
                        reinterpret_cast<cufftComplex*>(r->lattice), CUFFT_INVERSE));
    if (launch(r, "k_shiftLattice", {&r->lattice, &r->shifted, &acc})) return -1;
    if (launch(r, "k_calcGradientLattice", {&r->shifted, &r->forceXY})) return -1;
    if (launch(r, "k_forceMultiSampling", {&r->forceXY, &r->x, &r->y, &r->xo, &r->yo, &P, &acc})) return -1;
    return 0;
}

// One frame of the render chain on a density lattice already in r->acc.
int render_once(Ref* r) {
    if (launch(r, "k_copyAccumulatorIntoLattice", {&r->acc, &r->lattice})) return -1;
    if (launch(r, "k_getRealComponentOfLattice", {&r->lattice, &r->render1})) return -1;
    const unsigned smem = sizeof(float) * (3 + 32) * (3 + 32);  // BLUR_R = 3, TILE_SIZE = 32
    if (launch_shape(r, "k_calcBlurConvolution", dim3(32, 32), dim3(32, 32), smem, {&r->render1, &r->render2}))
        return -1;
    if (launch_shape(r, "k_resetMinMax", dim3(1), dim3(1), 0, {})) return -1;
    if (launch(r, "k_calcMinMax", {&r->render2})) return -1;
    if (launch_shape(r, "k_smoothMinMax", dim3(1), dim3(1), 0, {})) return -1;
    if (launch(r, "k_scaleWithMinMax", {&r->render2, &r->render1})) return -1;
    return 0;
}

void destroy(Ref* r) {
    if (r->st) cudaStreamSynchronize(r->st);
    if (r->plan) cufftDestroy(r->plan);
    for (void* p : {(void*)r->lattice, (void*)r->filter, (void*)r->deconv, (void*)r->forceXY, (void*)r->acc,
                    (void*)r->shifted, (void*)r->localForce, (void*)r->render1, (void*)r->render2, (void*)r->x, (void*)r->y, (void*)r->xo, (void*)r->yo,
                    (void*)r->m})
        cudaFree(p);
    if (r->mod) cuModuleUnload(r->mod);
    if (r->st) cudaStreamDestroy(r->st);
}

}  // namespace

extern "C" {

const char* ref_error(void) { return g_err.c_str(); }

void* ref_create(const char* ptx_path, int N, int cic, int P) {
    Ref* r = new Ref;
    if (create(r, ptx_path, N, cic, P)) {
        destroy(r);
        delete r;
        return nullptr;
    }
    return r;
}

void ref_destroy(void* h) {
    if (!h) return;
    destroy(static_cast<Ref*>(h));
    delete static_cast<Ref*>(h);
}

int ref_set_state(void* h, const float* x, const float* y, const float* xo, const float* yo, const float* m) {
    Ref* r = static_cast<Ref*>(h);
    const size_t b = size_t(r->P) * sizeof(float);
    RR_RT(cudaMemcpy(r->x, x, b, cudaMemcpyHostToDevice));
    RR_RT(cudaMemcpy(r->y, y, b, cudaMemcpyHostToDevice));
    RR_RT(cudaMemcpy(r->xo, xo, b, cudaMemcpyHostToDevice));
    RR_RT(cudaMemcpy(r->yo, yo, b, cudaMemcpyHostToDevice));
    RR_RT(cudaMemcpy(r->m, m, b, cudaMemcpyHostToDevice));
    return 0;
}

int ref_get_state(void* h, float* x, float* y, float* xo, float* yo) {
    Ref* r = static_cast<Ref*>(h);
    RR_RT(cudaStreamSynchronize(r->st));
    const size_t b = size_t(r->P) * sizeof(float);
    RR_RT(cudaMemcpy(x, r->x, b, cudaMemcpyDeviceToHost));
    RR_RT(cudaMemcpy(y, r->y, b, cudaMemcpyDeviceToHost));
    RR_RT(cudaMemcpy(xo, r->xo, b, cudaMemcpyDeviceToHost));
    RR_RT(cudaMemcpy(yo, r->yo, b, cudaMemcpyDeviceToHost));
    return 0;
}

// density (accumulator_d), potential (latticeShifted_d), force (latticeShiftedForceXY_d)
int ref_get_fields(void* h, float* density, float* potential, float* force_xy) {
    Ref* r = static_cast<Ref*>(h);
    RR_RT(cudaStreamSynchronize(r->st));
    const size_t NN = size_t(r->N) * r->N;
    RR_RT(cudaMemcpy(density, r->acc, NN * sizeof(float), cudaMemcpyDeviceToHost));
    RR_RT(cudaMemcpy(potential, r->shifted, NN * sizeof(float), cudaMemcpyDeviceToHost));
    RR_RT(cudaMemcpy(force_xy, r->forceXY, NN * sizeof(float2), cudaMemcpyDeviceToHost));
    return 0;
}

int ref_step(void* h, int nsteps) {
    Ref* r = static_cast<Ref*>(h);
    for (int i = 0; i < nsteps; ++i)
        if (step_once(r)) return -1;
    RR_RT(cudaStreamSynchronize(r->st));
    return 0;
}

// Render one display frame of `density` (N*N floats) into `frame` with the
// reference's render chain; the running min / max persist across calls.
int ref_render(void* h, const float* density, float* frame) {
    Ref* r = static_cast<Ref*>(h);
    const size_t NN = size_t(r->N) * r->N;
    RR_RT(cudaMemcpyAsync(r->acc, density, NN * sizeof(float), cudaMemcpyHostToDevice, r->st));
    if (render_once(r)) return -1;
    RR_RT(cudaMemcpyAsync(frame, r->render1, NN * sizeof(float), cudaMemcpyDeviceToHost, r->st));
    RR_RT(cudaStreamSynchronize(r->st));
    return 0;
}

// Device time per step (ms) over nsteps, CUDA events on the step stream.
float ref_time_steps(void* h, int nsteps) {
    Ref* r = static_cast<Ref*>(h);
    cudaEvent_t a, b;
    if (cudaEventCreate(&a) != cudaSuccess || cudaEventCreate(&b) != cudaSuccess) return -1.0f;
    cudaEventRecord(a, r->st);
    for (int i = 0; i < nsteps; ++i)
        if (step_once(r)) return -1.0f;
    cudaEventRecord(b, r->st);
    if (cudaEventSynchronize(b) != cudaSuccess) return -1.0f;
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, a, b);
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    return ms / float(nsteps > 0 ? nsteps : 1);
}

}  // extern "C"
