// fwi_aux.cu -- sm_103a kernels and C ABI of the routines around the
// gradient: gradient preconditioning (grad_precond_new5 + triangle2), the
// Butterworth band-pass (sfbandpass) and the cross-correlation misfit
// (XCORR1D).
//
// * triangle2 and sfbandpass are recursive along a line or a trace, so one
//   thread owns one line / trace and performs the reference's floating-point
//   operations in the reference's order, unfused (__f*_rn), giving results
//   bit-identical to triangle_smooth.c / butterworth_filter.c.
// * XCORR1D: one block per trace.  The two correlations the reference
//   evaluates with FFTs are direct sums here: zero-padded obs in shared
//   memory, each thread owns XB consecutive outputs and slides a register
//   window over obs while the other operand is broadcast.
#include "fwi_gb300.h"
#include "fwi_aux_kernels.cuh"

#include <cmath>
#include <cstring>
#include <vector>

using namespace fwi;

namespace fwi {

cudaError_t xcorr_setup()
{
    return cudaFuncSetAttribute(k_xcorr, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)XCORR_MAX_SMEM);
}

void launch_xcorr_traces(const float* obs, const float* syn, float* res, const float4* geo, float2* part, int ntr,
                         int nt, float omin, float omax, int slice, cudaStream_t st)
{
    FWI_LAUNCH(k_xcorr, (unsigned)ntr, XT, xcorr_smem_bytes(nt), st, obs, syn, res, geo, part, nt, omin, omax, slice);
}

void launch_xcorr_sum(const float2* part, int n, double* mis, cudaStream_t st)
{
    FWI_LAUNCH(k_xcorr_sum, 1, 1024, 0, st, part, n, mis);
}

}  // namespace fwi

namespace {

// Device buffers of one standalone call, freed on every exit path.
struct Scratch {
    std::vector<void*> ptrs;
    ~Scratch()
    {
        for (void* p : ptrs) cudaFree(p);
    }
    template <class T> T* alloc(size_t n)
    {
        T* p = nullptr;
        if (cudaMalloc(&p, sizeof(T) * (n ? n : 1)) != cudaSuccess) { cudaGetLastError(); return nullptr; }
        ptrs.push_back(p);
        return p;
    }
};

int device_ready()
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) { cudaGetLastError(); return FWI_ERR_NODEVICE; }
    cudaDeviceProp prop{};
    if (cudaGetDeviceProperties(&prop, dev) != cudaSuccess || prop.major != 10 || prop.minor != 3) {
        cudaGetLastError();
        return FWI_ERR_NODEVICE;
    }
    return FWI_OK;
}

#define AUX_CK(call)                                                 \
    do {                                                             \
        if ((call) != cudaSuccess) { cudaGetLastError(); return FWI_ERR_CUDA; } \
    } while (0)

}  // namespace

extern "C" {

int fwi_grad_precond(float* body, int mnx, int mnz, float perc, int rectx1, int repeat1, int rectx2, int repeat2,
                     float alpha_grad, const int* bottom)
{
    if (!body || !bottom || mnx < 1 || mnz < 1 || rectx1 < 1 || rectx2 < 1 || repeat1 < 0 || repeat2 < 0)
        return FWI_ERR_ARG;
    if (int s = device_ready()) return s;
    const size_t n = (size_t)mnx * mnz;
    Scratch S;
    float* a = S.alloc<float>(n);
    float* b = S.alloc<float>(n);
    int* bot = S.alloc<int>(mnx);
    float* mm = S.alloc<float>(2);
    const int nlines = mnx > mnz ? mnx : mnz, nmax = nlines, rmax = rectx1 > rectx2 ? rectx1 : rectx2;
    float* work = S.alloc<float>((size_t)nlines * tri_work_floats(rmax, nmax));
    if (!a || !b || !bot || !mm || !work) return FWI_ERR_NOMEM;
    cudaStream_t st = nullptr;
    AUX_CK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    struct StreamGuard { cudaStream_t s; ~StreamGuard() { cudaStreamDestroy(s); } } guard{st};
    AUX_CK(cudaMemcpyAsync(a, body, sizeof(float) * n, cudaMemcpyHostToDevice, st));
    AUX_CK(cudaMemcpyAsync(bot, bottom, sizeof(int) * mnx, cudaMemcpyHostToDevice, st));
    // clip to perc * (min, max) (grad_prec.c:16-35)
    FWI_LAUNCH(k_minmax, 1, 1024, 0, st, a, (long long)n, mm);
    if (perc != 0) FWI_LAUNCH(k_clip, (unsigned)((n + 255) / 256), 256, 0, st, a, (long long)n, mm, perc);
    // b = triangle2(rectx1, rectx1, repeat1) of a, masked, then triangle2(rectx2, rectx2, repeat2) in place
    AUX_CK(cudaMemcpyAsync(b, a, sizeof(float) * n, cudaMemcpyDeviceToDevice, st));
    launch_triangle2(b, mnx, mnz, rectx1, rectx1, repeat1, work, st);
    FWI_LAUNCH(k_mask_bottom, (unsigned)((n + 255) / 256), 256, 0, st, b, mnx, mnz, bot);
    launch_triangle2(b, mnx, mnz, rectx2, rectx2, repeat2, work, st);
    FWI_LAUNCH(k_scale, (unsigned)((n + 255) / 256), 256, 0, st, b, (long long)n, alpha_grad);
    AUX_CK(cudaGetLastError());
    AUX_CK(cudaMemcpyAsync(body, b, sizeof(float) * n, cudaMemcpyDeviceToHost, st));
    AUX_CK(cudaStreamSynchronize(st));
    return FWI_OK;
}

int fwi_bandpass(const float* indat, int nt, int nr, float dt, int phase, int nphi, int nplo, float fhi, float flo,
                 float* outdat)
{
    if (!indat || !outdat || nt < 1 || nr < 1 || !(dt > 0)) return FWI_ERR_ARG;
    if (!(flo >= 0)) return FWI_ERR_ARG;                       // the reference exits on flo < 0
    if (nphi > BUTTER_MAX_ORDER || nplo > BUTTER_MAX_ORDER) return FWI_ERR_ARG;
    ButterPair bp;
    butter_pair(dt, phase, nphi, nplo, fhi, flo, &bp);
    if (int s = device_ready()) return s;
    Scratch S;
    const size_t n = (size_t)nt * nr;
    float* x = S.alloc<float>(n);
    if (!x) return FWI_ERR_NOMEM;
    cudaStream_t st = nullptr;
    AUX_CK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    struct StreamGuard { cudaStream_t s; ~StreamGuard() { cudaStreamDestroy(s); } } guard{st};
    AUX_CK(cudaMemcpyAsync(x, indat, sizeof(float) * n, cudaMemcpyHostToDevice, st));
    FWI_LAUNCH(k_bandpass, (unsigned)((nr + 127) / 128), 128, 0, st, x, nt, nr, bp);
    AUX_CK(cudaGetLastError());
    AUX_CK(cudaMemcpyAsync(outdat, x, sizeof(float) * n, cudaMemcpyDeviceToHost, st));
    AUX_CK(cudaStreamSynchronize(st));
    return FWI_OK;
}

int fwi_xcorr1d(const float* obs, const float* syn, int nr, int nt, const float* sr_xyz, float offset_min,
                float offset_max, int slice, float* misfit, float* res)
{
    if (!obs || !syn || !sr_xyz || !misfit || !res || nr < 1 || nt < 1 || (slice != 0 && slice != 1))
        return FWI_ERR_ARG;
    if (xcorr_smem_bytes(nt) > XCORR_MAX_SMEM) return FWI_ERR_ARG;
    if (int s = device_ready()) return s;
    Scratch S;
    const size_t n = (size_t)nt * nr;
    float* o = S.alloc<float>(n);
    float* s = S.alloc<float>(n);
    float* r = S.alloc<float>(n);
    float4* geo = S.alloc<float4>(nr);
    float2* part = S.alloc<float2>(nr);
    double* mis = S.alloc<double>(2);
    if (!o || !s || !r || !geo || !part || !mis) return FWI_ERR_NOMEM;
    std::vector<float4> g(nr);
    for (int i = 0; i < nr; ++i) g[i] = make_float4(sr_xyz[0], sr_xyz[1], sr_xyz[2 + 2 * i], sr_xyz[3 + 2 * i]);
    cudaStream_t st = nullptr;
    AUX_CK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    struct StreamGuard { cudaStream_t s; ~StreamGuard() { cudaStreamDestroy(s); } } guard{st};
    AUX_CK(cudaMemcpyAsync(o, obs, sizeof(float) * n, cudaMemcpyHostToDevice, st));
    AUX_CK(cudaMemcpyAsync(s, syn, sizeof(float) * n, cudaMemcpyHostToDevice, st));
    AUX_CK(cudaMemcpyAsync(geo, g.data(), sizeof(float4) * nr, cudaMemcpyHostToDevice, st));
    AUX_CK(xcorr_setup());
    launch_xcorr_traces(o, s, r, geo, part, nr, nt, offset_min, offset_max, slice, st);
    launch_xcorr_sum(part, nr, mis, st);
    AUX_CK(cudaGetLastError());
    double m[2];
    AUX_CK(cudaMemcpyAsync(m, mis, sizeof(m), cudaMemcpyDeviceToHost, st));
    AUX_CK(cudaMemcpyAsync(res, r, sizeof(float) * n, cudaMemcpyDeviceToHost, st));
    AUX_CK(cudaStreamSynchronize(st));
    misfit[0] = (float)m[0];
    misfit[1] = (float)m[1];
    return FWI_OK;
}

}  // extern "C"
