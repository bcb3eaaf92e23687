// cpu_emu.h -- host emulation of the small part of CUDA that the engine uses,
// for memory-safety checks of the kernels on a machine without a GPU.
//
// Compiling fwi_engine.cu as C++ with -DFWI_CPU_EMU (build.py build_emu)
// runs every kernel on the CPU: the blocks of a launch execute one after
// another, each on a pool of OS threads (one per CUDA thread), __syncthreads
// is a barrier of that pool, __shared__ arrays are block-wide statics and
// every device allocation is an exact-size heap block, so AddressSanitizer
// reports any access outside a buffer.  Timing, streams and graphs are
// no-ops; results are bit-identical to a sequential execution of the
// kernels.  Diagnostics only: the product build never defines FWI_CPU_EMU.
#pragma once
#ifdef FWI_CPU_EMU

#include <algorithm>
#include <atomic>
#include <barrier>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <mutex>
#include <thread>
#include <tuple>
#include <vector>

#define __global__
#define __device__
#define __host__
#define __forceinline__ inline
#define __launch_bounds__(...)
#define __grid_constant__
#define __shared__ static
#define __align__(n) __attribute__((aligned(n)))
#define FWI_DYN_SMEM(name) unsigned char* name = fwi_emu::dyn_smem()

struct dim3 {
    unsigned x = 1, y = 1, z = 1;
    dim3(unsigned a = 1, unsigned b = 1, unsigned c = 1) : x(a), y(b), z(c) {}
};
struct int2 { int x, y; };
struct alignas(8) float2 { float x, y; };
struct alignas(16) float4 { float x, y, z, w; };
inline int2 make_int2(int a, int b) { return int2{a, b}; }
inline float2 make_float2(float a, float b) { return float2{a, b}; }
inline float4 make_float4(float a, float b, float c, float d) { return float4{a, b, c, d}; }

inline thread_local dim3 threadIdx, blockIdx, blockDim, gridDim;

using std::max;
using std::min;
inline float __fmul_rn(float a, float b) { return a * b; }
inline float __fadd_rn(float a, float b) { return a + b; }
inline float __fsub_rn(float a, float b) { return a - b; }
inline float __fdiv_rn(float a, float b) { return a / b; }
template <class T> inline T __ldg(const T* p) { return *p; }
template <class T> inline T __ldcg(const T* p) { return *p; }
template <class T> inline void __stcg(T* p, T v) { *p = v; }
inline float atomicAdd(float* p, float v) { return std::atomic_ref<float>(*p).fetch_add(v); }
inline unsigned atomicMax(unsigned* p, unsigned v)
{
    unsigned cur = std::atomic_ref<unsigned>(*p).load();
    while (cur < v && !std::atomic_ref<unsigned>(*p).compare_exchange_weak(cur, v)) {}
    return cur;
}
inline unsigned __float_as_uint(float f) { unsigned u; std::memcpy(&u, &f, 4); return u; }
inline float __uint_as_float(unsigned u) { float f; std::memcpy(&f, &u, 4); return f; }
// 16-bit storage types of checkpoints: IEEE binary16 through the compiler's
// _Float16 (round to nearest even), bfloat16 as the upper half of a float
// rounded to nearest even by the usual bias of 0x7fff plus the kept LSB.
struct __half { _Float16 v; };
struct __nv_bfloat16 { unsigned short b; };
inline __half __float2half_rn(float f) { return __half{(_Float16)f}; }
inline float __half2float(__half h) { return (float)h.v; }
inline __nv_bfloat16 __float2bfloat16_rn(float f)
{
    const unsigned u = __float_as_uint(f);
    return __nv_bfloat16{(unsigned short)((u + 0x7fffu + ((u >> 16) & 1u)) >> 16)};
}
inline float __bfloat162float(__nv_bfloat16 h) { return __uint_as_float((unsigned)h.b << 16); }
inline int atomicCAS(int* p, int cmp, int val)
{
    std::atomic_ref<int>(*p).compare_exchange_strong(cmp, val);
    return cmp;
}

namespace fwi_emu {

struct Pool {
    int nthreads = 0;
    std::barrier<>* bar = nullptr;                 // __syncthreads
    std::vector<std::barrier<>*> warp_bar;         // __shfl_*_sync
    std::vector<double> shfl;                      // one slot per thread
    std::function<void()> body;
    unsigned long long epoch = 0;
    int done = 0;
    int gen = 0;                                   // workers of an older generation exit
    int exiting = 0;                               // old workers that have not exited yet
    std::mutex m;
    std::condition_variable cv, cv_done;
    dim3 bdim, gdim, bidx;
};

inline Pool& pool()
{
    static Pool* p = new Pool;   // never destroyed: idle workers may still wait on it at exit
    return *p;
}

inline thread_local std::vector<unsigned char>* tl_dyn = nullptr;
inline std::vector<unsigned char>& dyn_buf()
{
    static std::vector<unsigned char> b;
    return b;
}
inline unsigned char* dyn_smem() { return dyn_buf().data(); }

inline void worker(int tid, int gen, unsigned long long seen)
{
    Pool& P = pool();
    for (;;) {
        std::function<void()> body;
        {
            std::unique_lock<std::mutex> lk(P.m);
            P.cv.wait(lk, [&] { return P.gen != gen || P.epoch != seen; });
            if (P.gen != gen) {
                if (--P.exiting == 0) P.cv_done.notify_all();
                return;
            }
            seen = P.epoch;
            body = P.body;
            blockDim = P.bdim;
            gridDim = P.gdim;
            blockIdx = P.bidx;
        }
        threadIdx = dim3(tid % P.bdim.x, (tid / P.bdim.x) % P.bdim.y, tid / (P.bdim.x * P.bdim.y));
        body();
        {
            std::lock_guard<std::mutex> lk(P.m);
            if (++P.done == P.nthreads) P.cv_done.notify_all();
        }
    }
}

// A pool of n workers; the workers of a pool of another size exit first.
inline void ensure_pool(int n)
{
    Pool& P = pool();
    if (P.nthreads == n) return;
    if (P.nthreads) {
        std::unique_lock<std::mutex> lk(P.m);
        P.exiting = P.nthreads;
        ++P.gen;
        P.cv.notify_all();
        P.cv_done.wait(lk, [&] { return P.exiting == 0; });
        delete P.bar;
        for (auto* b : P.warp_bar) delete b;
        P.warp_bar.clear();
    }
    P.nthreads = n;
    P.bar = new std::barrier<>(n);
    for (int w = 0; w < (n + 31) / 32; ++w) P.warp_bar.push_back(new std::barrier<>(std::min(32, n - 32 * w)));
    P.shfl.assign(n, 0.0);
    for (int t = 0; t < n; ++t) {
        std::thread th(worker, t, P.gen, P.epoch);
        th.detach();           // idle workers end with the process
    }
}

// Runs kernel(args...) over the grid, block after block.
template <class... KArgs, class... Args>
void launch(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, Args&&... args)
{
    const int n = (int)(block.x * block.y * block.z);
    ensure_pool(n);
    Pool& P = pool();
    dyn_buf().assign(smem ? smem : 1, 0);
    auto tuple_args = std::make_tuple(args...);
    for (unsigned bz = 0; bz < grid.z; ++bz)
        for (unsigned by = 0; by < grid.y; ++by)
            for (unsigned bx = 0; bx < grid.x; ++bx) {
                {
                    std::lock_guard<std::mutex> lk(P.m);
                    P.body = [&] { std::apply([&](auto&... a) { kernel(a...); }, tuple_args); };
                    P.bdim = block;
                    P.gdim = grid;
                    P.bidx = dim3(bx, by, bz);
                    P.done = 0;
                    ++P.epoch;
                }
                P.cv.notify_all();
                std::unique_lock<std::mutex> lk(P.m);
                P.cv_done.wait(lk, [&] { return P.done == P.nthreads; });
            }
}

inline int linear_tid() { return (int)(threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z)); }

}  // namespace fwi_emu

inline void __syncthreads() { fwi_emu::pool().bar->arrive_and_wait(); }

template <class T> inline T shfl_xor_emu(T v, int lane_mask);
inline double __shfl_xor_sync(unsigned, double v, int lane_mask) { return shfl_xor_emu<double>(v, lane_mask); }
inline float __shfl_xor_sync(unsigned, float v, int lane_mask) { return (float)shfl_xor_emu<double>(v, lane_mask); }
template <class T> inline T shfl_xor_emu(T v, int lane_mask)
{
    fwi_emu::Pool& P = fwi_emu::pool();
    const int t = fwi_emu::linear_tid(), w = t / 32;
    P.shfl[t] = v;
    P.warp_bar[w]->arrive_and_wait();
    const int src = (t & ~31) | ((t & 31) ^ lane_mask);
    const double r = (src < P.nthreads) ? P.shfl[src] : v;
    P.warp_bar[w]->arrive_and_wait();
    return r;
}

// ---- runtime API -----------------------------------------------------------
typedef int cudaError_t;
typedef void* cudaStream_t;
typedef void* cudaEvent_t;
typedef void* cudaGraph_t;
typedef void* cudaGraphExec_t;
enum { cudaSuccess = 0, cudaErrorInvalidDevice = 101, cudaErrorNotSupported = 801 };
enum cudaMemcpyKind { cudaMemcpyHostToDevice, cudaMemcpyDeviceToHost, cudaMemcpyDeviceToDevice };
enum { cudaStreamNonBlocking = 1, cudaEventDisableTiming = 2 };
enum cudaStreamCaptureMode { cudaStreamCaptureModeThreadLocal };
enum cudaStreamCaptureStatus { cudaStreamCaptureStatusNone, cudaStreamCaptureStatusActive };
enum cudaFuncAttribute { cudaFuncAttributeMaxDynamicSharedMemorySize };
enum cudaDeviceAttr { cudaDevAttrMultiProcessorCount };
struct cudaDeviceProp { int major = 10, minor = 3; };

inline const char* cudaGetErrorString(cudaError_t e) { return e ? "emulation: not supported" : "no error"; }
inline cudaError_t cudaGetLastError() { return cudaSuccess; }
inline cudaError_t cudaPeekAtLastError() { return cudaSuccess; }
inline cudaError_t cudaStreamIsCapturing(cudaStream_t, cudaStreamCaptureStatus* c) { *c = cudaStreamCaptureStatusNone; return cudaSuccess; }
inline cudaError_t cudaGetDeviceCount(int* n) { *n = 1; return cudaSuccess; }
inline cudaError_t cudaDeviceGetAttribute(int* v, cudaDeviceAttr, int) { *v = 4; return cudaSuccess; }   // 4 emulated SMs
inline cudaError_t cudaGetDeviceProperties(cudaDeviceProp* p, int) { *p = cudaDeviceProp{}; return cudaSuccess; }
inline cudaError_t cudaSetDevice(int) { return cudaSuccess; }
inline cudaError_t cudaGetDevice(int* d) { *d = 0; return cudaSuccess; }
template <class T> inline cudaError_t cudaGetSymbolAddress(void** p, T& sym) { *p = (void*)&sym; return cudaSuccess; }
template <class T> inline cudaError_t cudaMemcpyToSymbol(T& sym, const void* src, size_t n) { std::memcpy(&sym, src, n); return cudaSuccess; }
template <class T> inline cudaError_t cudaMemcpyFromSymbol(void* dst, const T& sym, size_t n) { std::memcpy(dst, &sym, n); return cudaSuccess; }
template <class T> inline cudaError_t cudaMalloc(T** p, size_t n)
{
    *p = (T*)std::malloc(n ? n : 1);
    return *p ? cudaSuccess : 2;
}
inline cudaError_t cudaFree(void* p) { std::free(p); return cudaSuccess; }
inline cudaError_t cudaMemGetInfo(size_t* fr, size_t* tot) { *fr = *tot = (size_t)1 << 34; return cudaSuccess; }
inline cudaError_t cudaMemcpy(void* d, const void* s, size_t n, cudaMemcpyKind) { std::memcpy(d, s, n); return cudaSuccess; }
inline cudaError_t cudaMemcpyAsync(void* d, const void* s, size_t n, cudaMemcpyKind, cudaStream_t) { std::memcpy(d, s, n); return cudaSuccess; }
inline cudaError_t cudaMemset(void* d, int v, size_t n) { std::memset(d, v, n); return cudaSuccess; }
inline cudaError_t cudaMemsetAsync(void* d, int v, size_t n, cudaStream_t) { std::memset(d, v, n); return cudaSuccess; }
inline cudaError_t cudaStreamCreateWithFlags(cudaStream_t* s, int) { *s = (void*)0x1; return cudaSuccess; }
inline cudaError_t cudaStreamDestroy(cudaStream_t) { return cudaSuccess; }
inline cudaError_t cudaStreamCreateWithPriority(cudaStream_t* s, int, int) { *s = (void*)0x1; return cudaSuccess; }
inline cudaError_t cudaDeviceGetStreamPriorityRange(int* least, int* greatest) { *least = 0; *greatest = -5; return cudaSuccess; }
inline cudaError_t cudaStreamSynchronize(cudaStream_t) { return cudaSuccess; }
inline cudaError_t cudaEventCreate(cudaEvent_t* e) { *e = (void*)0x1; return cudaSuccess; }
inline cudaError_t cudaEventCreateWithFlags(cudaEvent_t* e, int) { *e = (void*)0x1; return cudaSuccess; }
inline cudaError_t cudaStreamWaitEvent(cudaStream_t, cudaEvent_t, int) { return cudaSuccess; }
inline cudaError_t cudaEventDestroy(cudaEvent_t) { return cudaSuccess; }
inline cudaError_t cudaEventRecord(cudaEvent_t, cudaStream_t) { return cudaSuccess; }
inline cudaError_t cudaEventElapsedTime(float* ms, cudaEvent_t, cudaEvent_t) { *ms = 0.f; return cudaSuccess; }
template <class F> inline cudaError_t cudaFuncSetAttribute(F, cudaFuncAttribute, int) { return cudaSuccess; }
inline cudaError_t cudaStreamBeginCapture(cudaStream_t, cudaStreamCaptureMode) { return cudaErrorNotSupported; }
inline cudaError_t cudaStreamEndCapture(cudaStream_t, cudaGraph_t*) { return cudaErrorNotSupported; }
inline cudaError_t cudaGraphInstantiate(cudaGraphExec_t*, cudaGraph_t, int) { return cudaErrorNotSupported; }
inline cudaError_t cudaGraphLaunch(cudaGraphExec_t, cudaStream_t) { return cudaErrorNotSupported; }
inline cudaError_t cudaGraphDestroy(cudaGraph_t) { return cudaSuccess; }
inline cudaError_t cudaGraphExecDestroy(cudaGraphExec_t) { return cudaSuccess; }

#define FWI_LAUNCH(kernel, grid, block, smem, stream, ...) fwi_emu::launch(kernel, grid, block, smem, __VA_ARGS__)
#define FWI_LAUNCH_PDL(kernel, grid, block, smem, stream, ...) fwi_emu::launch(kernel, grid, block, smem, __VA_ARGS__)

#else  // the real CUDA build

#define FWI_DYN_SMEM(name) extern __shared__ __align__(16) unsigned char name[]
#define FWI_LAUNCH(kernel, grid, block, smem, stream, ...) kernel<<<grid, block, smem, stream>>>(__VA_ARGS__)
// A launch that may start while the previous kernel on its stream finishes
// (programmatic dependent launch); the kernel waits for that kernel's results
// with griddepcontrol.wait before it reads them (pdl_begin).
template <typename... KArgs, typename... Args>
inline cudaError_t fwi_launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t stream,
                                  Args... args)
{
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = stream;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, static_cast<KArgs>(args)...);
}
#define FWI_LAUNCH_PDL(kernel, grid, block, smem, stream, ...) fwi_launch_pdl(kernel, grid, block, smem, stream, __VA_ARGS__)

#endif
