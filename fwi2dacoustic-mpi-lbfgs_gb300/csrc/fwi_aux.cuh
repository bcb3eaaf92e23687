// fwi_aux.cuh -- launchers of the routines around the gradient whose
// kernels live in fwi_aux.cu (fwi_aux_kernels.cuh): the XCORR misfit, used by
// fwi_aux.cu's standalone entry point and by the engine's misfit phase.
#pragma once
#ifdef FWI_CPU_EMU
#include "cpu_emu.h"
#else
#include <cuda_runtime.h>
#include "cpu_emu.h"
#endif
#include <cstddef>

namespace fwi {

constexpr int XB = 7;                       // XCORR outputs per thread (odd: conflict-free window loads)
constexpr int XT = 256;                     // XCORR threads per trace block
constexpr size_t XCORR_MAX_SMEM = 227 * 1024;

// Dynamic shared memory of one XCORR trace block: 64 doubles of reduction
// scratch, obs zero-padded on both sides (3 nt + 2 XB + 2 floats), syn, and
// the correlation / its gradient (nt floats each).
inline size_t xcorr_smem_bytes(int nt) { return sizeof(float) * ((size_t)5 * nt + 2 * XB + 2) + 64 * sizeof(double); }

// Allows XCORR blocks up to XCORR_MAX_SMEM bytes of shared memory (call
// outside stream capture, before the first launch).
cudaError_t xcorr_setup();

// XCORR1D terms of ntr traces of nt samples ([ntr][nt] obs, syn -> res;
// geo[ntr] = source x, z, receiver x, z; part[ntr] = {misfit[0] term,
// alpha}); slice 0 "middle", 1 "leading".  Launches only (capture-safe).
void launch_xcorr_traces(const float* obs, const float* syn, float* res, const float4* geo, float2* part, int ntr,
                         int nt, float omin, float omax, int slice, cudaStream_t st);

// mis[0] = sum of part[].x, mis[1] = sum of part[].y over n traces (FP64).
void launch_xcorr_sum(const float2* part, int n, double* mis, cudaStream_t st);

}  // namespace fwi
