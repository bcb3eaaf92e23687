// fwi_engine.cu -- host side of the C ABI declared in include/fwi_gb300.h.
//
// Owns the device state of one batch of shots and drives the per-step
// kernels of fwi_kernels.cuh.  Replaces, for the hot path, the per-rank plan
// setup fwi_init (fwi_2d.c:139-396) and the missing per-shot driver
// grad4_1shot (header.h:283): all shots of an iteration live on one GPU and
// every time step of every shot is one launch (grid.z = shot).
#include "fwi_gb300.h"
#include "fwi_kernels.cuh"
#include "fwi_kernels8.cuh"
#include "fwi_aux.cuh"
#ifndef FWI_CPU_EMU
#include <cudaTypedefs.h>
#endif

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstddef>
#include <cstdlib>
#include <mutex>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

using namespace fwi;

// Scratch of fwi_l2_misfit_noalloc: one FP64 sum of squares per trace.  It
// lives in the library image, so every device that loads the library holds
// these 512 KB until the process exits; no call ever allocates.
static __device__ __align__(256) double g_noalloc_trace_sums[FWI_NOALLOC_MAX_TRACES];

namespace {

constexpr int kVersion = 1;
// Shots of one batch: the stencil launches put the shot in blockIdx.z.
constexpr int MAX_SHOTS = 65535;

inline long long round_up(long long a, long long b) { return (a + b - 1) / b * b; }

// CPML damping profile on 2*npml+1 half-cell nodes, cpml_coe (fwi_2d.c:110-137)
// with pml_base.dim = 2.  The reference mixes float locals with double libm
// calls (log, exp) and double constants; the same promotions are kept here so
// that the profile is bit-identical to the reference's.
void cpml_profile(float* a0, float* b0, int npml, float d, float dt, float maxF, float maxV, float coefR)
{
    const float half = d * 0.5;
    const int npower = 2;
    const float width = npml * d;
    const float pif0 = 3.141592654 * maxF;          // PI as fwi_sys.h:1 defines it
    const float slope = pif0 / width;
    const float d0 = -(npower + 1) * maxV * std::log((double)coefR) / (2.0 * width);
    for (int i = 0; i < 2 * npml + 1; ++i) {
        float damp = (1.0 - i * half / width);
        damp *= damp;
        damp *= d0;
        const float alpha = slope * (i * half);
        b0[i] = (float)std::exp((double)(-(damp + alpha) * dt));
        a0[i] = (float)(damp / (damp + alpha) * (b0[i] - 1.0));
    }
}

// FD coefficients as fwi_init sets them (fwi_2d.c:304-314): the optimized
// 4th-order staggered pair (1.129042, -0.04301412) scaled by 1/h.
void fd_coefficients(float dx, float dz, float out[8])
{
    const float ix = 1.0 / dx, iz = 1.0 / dz;
    out[0] = 0.1129042e1 * ix;  out[1] = -0.4301412e-1 * ix;  out[2] = ix;
    out[3] = 0.1129042e1 * iz;  out[4] = -0.4301412e-1 * iz;  out[5] = iz;
    out[6] = iz / 840.0;        out[7] = iz / 24.0;
}

// Cell of a position in metres, fwi_2d.c:363-364.
inline void cell_of(float x, float z, float dx, float dz, int* ix, int* iz)
{
    *ix = (int)std::round(x / dx);
    *iz = (int)std::round(z / dz - 0.5);
}

}  // namespace

struct fwi_ctx {
    fwi_config cfg{};
    cudaStream_t own = nullptr;    // the context's stream
    cudaStream_t st = nullptr;     // stream in use (own, or the caller's)
    cudaEvent_t ev[8]{};           // [0,1] forward, [2,3] backward, [4,5] misfit, [6,7] whole call
    // The general-tile classes of a step run on side streams, forked from and
    // joined back into st around every step, concurrently with the interior
    // tiles (they write disjoint cells and read the same inputs).  A captured
    // graph keeps them as parallel branches.
    cudaStream_t side[3]{};
    cudaEvent_t fork_ev = nullptr, join_ev[3]{};
    cudaStream_t samp_st = nullptr;                // receiver sampling, off the forward's critical path
    cudaEvent_t step_ev = nullptr, samp_ev[2]{}, samp_done = nullptr;
    bool samp_pending[2] = {false, false};         // a sample of that step parity is not yet waited for
    bool samp_used = false;                        // samp_st has work in this forward pass
    int nsm = 1;                                   // streaming multiprocessors of the device
#ifdef FWI_TIMELINE
    unsigned long long* tl_d = nullptr;            // block timeline (diagnostics build), written out on destroy
    std::string tl_out;
#endif
    cudaStream_t obs_st = nullptr;                 // fwi_gradient_obs: observed-trace upload under the forward phase
    cudaEvent_t obs_ev = nullptr;
    cudaGraph_t graph[3]{};        // captured phases (use_graph): forward, misfit, backward
    cudaGraphExec_t gexec[3]{};
    long long graph_launches[3]{};
    Geo g{};
    Coef c{};
    PsiLayout pl{};
    int rows_alloc = 0;
    long long origin = 0;          // floats from a shot block's start to (row 0, col 0)
    float* K = nullptr;            // one shot block
    float* vel = nullptr;          // [nz][nx]
    float* pmlc = nullptr;         // 8 * (2*npml+1)
    // per-shot state
    int nshots = 0;
    int nt_run = 0;
    float* F = nullptr;            // 2 x nshots x fstride (forward field / rebuild)
    float* A = nullptr;            // 2 x nshots x fstride (adjoint)
    float* Gacc = nullptr;         // nshots x fstride
    float* psiF = nullptr;         // 2 x nshots x pl.stride
    float* psiA = nullptr;
    float* ring = nullptr;
    float* syn = nullptr;
    float* res = nullptr;
    float* obs = nullptr;
    float* wav = nullptr;
    double* grad = nullptr;
    float* gradf = nullptr;
    double* partial = nullptr;
    double* mis = nullptr;
    ShotDev* shots_d = nullptr;
    RecSample* samp_d = nullptr;   // receivers, slot order (forward sampling)
    RecDev* recs_d = nullptr;      // receivers grouped by tile (backward injection)
    int* rtile_d = nullptr;        // per-slot, per-tile CSR of recs_d
    int2* gen_d = nullptr;         // tiles of the general path, grouped by class (GX only, GZ only, both)
    int* err_d = nullptr;          // set by a kernel whose tile copy timed out (StepParams::err)
    TensorMap tm_F[2], tm_A[2];    // TMA maps of the two halves of F (p) and A (b)
    int ngen = 0;
    int gen_off[4] = {};           // class c occupies gen_d[gen_off[c], gen_off[c + 1])
    int ftx0 = 0, ftx1 = 0, ftz0 = 0, ftz1 = 0;   // interior tile rectangle
    int gen_arith = 0;             // gen_d agrees with gen_tile_at
    std::vector<int> samp_off;                    // per-slot ranges (nshots + 1)
    std::vector<int> nt_slot;      // nt of each slot, descending
    long long nsamples = 0;
    int npartial = 0;
    // misfit of fwi_gradient; XCORR works per shot on its traces
    fwi_misfit msf{};
    float4* geo_d = nullptr;       // per trace: source x, z, receiver x, z (metres)
    float2* xpart_d = nullptr;     // per trace: XCORR misfit terms
    std::vector<long long> shot_syn_off;          // per shot (input order): first sample of its traces
    std::vector<int> shot_tr0, shot_nr, shot_nt0; // first trace, traces, samples per trace
    int ntraces = 0;
    bool have_model = false, have_obs = false, have_fwd = false;
    bool broken = false;           // a tile copy timed out: device state undefined, no further work
    // forward-field storage (FWI_STORE_*): strips of every step, or checkpoints
    // of the forward state at segment starts plus the strips of one segment
    int store = FWI_STORE_STRIPS;
    int seg = 0, nseg = 1;         // snapshots: segment length and count (strips: one segment)
    int nsnap = 0;                 // checkpoints held: those of segments 1 .. nseg-2
    void* snapP = nullptr;         // [nsnap][nshots][2][fstride] in snap_precision
    float* snapPsi = nullptr;      // [nsnap][nshots][pl.stride]
    unsigned* snapAmax = nullptr;  // [nsnap][nshots][2] absmax bits (F16 / BF16)
    long long store_bytes = 0;
    fwi_tuning tune{};             // launch tuning in use, every field resolved (fwi_set_tuning)
    // FD order: M = 2 (the reference's 4th order) or M = 4 (8th order, fwi_kernels8.cuh)
    int M = 2, S = 3;              // half order, strip width 2M-1
    float* X8 = nullptr;           // M = 4: u, v (or their adjoints), rebuild u, v: 4 x nshots x fstride
    RecCell8* cells8_d = nullptr;  // M = 4: receiver cells of the backward injection, by slot
    long long* rec8_d = nullptr;   // M = 4: syn offsets of the receivers, grouped by cell
    int ncell8 = 0;
    std::vector<int> cell8_off;    // M = 4: slot k's cells are cells8_d[cell8_off[k], cell8_off[k + 1])
    size_t bytes_model = 0, bytes_shots = 0;
    std::string err;
    fwi_stats stats{};
};

namespace {

int fail(fwi_ctx* x, int code, const std::string& msg)
{
    if (x) x->err = msg;
    return code;
}

int cuda_fail(fwi_ctx* x, cudaError_t e, const char* what)
{
    return fail(x, FWI_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

#define CK(call)                                                       \
    do {                                                               \
        cudaError_t e_ = (call);                                       \
        if (e_ != cudaSuccess) return cuda_fail(x, e_, #call);         \
    } while (0)

template <class T>
int dalloc(fwi_ctx* x, T** p, size_t n, size_t* acc)
{
    if (n == 0) n = 1;
    cudaError_t e = cudaMalloc((void**)p, n * sizeof(T));
    if (e != cudaSuccess) {
        *p = nullptr;
        cudaGetLastError();
        return fail(x, FWI_ERR_NOMEM, std::string("cudaMalloc of ") + std::to_string(n * sizeof(T)) + " bytes failed");
    }
    *acc += n * sizeof(T);
    return FWI_OK;
}

void drop_graph(fwi_ctx* x)
{
    for (int i = 0; i < 3; ++i) {
        if (x->gexec[i]) cudaGraphExecDestroy(x->gexec[i]);
        if (x->graph[i]) cudaGraphDestroy(x->graph[i]);
        x->gexec[i] = nullptr;
        x->graph[i] = nullptr;
    }
}

void free_shots(fwi_ctx* x)
{
    drop_graph(x);
    void* ps[] = {x->F, x->A, x->Gacc, x->psiF, x->psiA, x->ring, x->syn, x->res, x->obs, x->wav,
                  x->shots_d, x->samp_d, x->recs_d, x->rtile_d, x->partial, x->mis, x->geo_d, x->xpart_d,
                  x->snapP, x->snapPsi, x->snapAmax, x->X8, x->cells8_d, x->rec8_d};
    for (void* p : ps) if (p) cudaFree(p);
    x->snapP = nullptr; x->snapPsi = nullptr; x->snapAmax = nullptr;
    x->X8 = nullptr; x->cells8_d = nullptr; x->rec8_d = nullptr; x->ncell8 = 0;
    x->store = FWI_STORE_STRIPS; x->seg = 0; x->nseg = 1; x->nsnap = 0; x->store_bytes = 0;
    x->F = x->A = x->Gacc = x->psiF = x->psiA = x->ring = x->syn = x->res = x->obs = x->wav = nullptr;
    x->shots_d = nullptr; x->samp_d = nullptr; x->recs_d = nullptr; x->rtile_d = nullptr;
    x->partial = nullptr; x->mis = nullptr; x->geo_d = nullptr; x->xpart_d = nullptr;
    x->shot_syn_off.clear(); x->shot_tr0.clear(); x->shot_nr.clear(); x->shot_nt0.clear();
    x->ntraces = 0;
    x->samp_off.clear();
    x->nshots = 0; x->nt_run = 0; x->nsamples = 0; x->bytes_shots = 0;
    x->nt_slot.clear();
    x->have_obs = x->have_fwd = false;
}

StepParams base_params(const fwi_ctx* x)
{
    StepParams P{};
    P.g = x->g;
    P.c = x->c;
    P.K = x->K + x->origin;
    P.pmlc = x->pmlc;
    P.pl = x->pl;
    P.shots = x->shots_d;
    P.gen_tiles = x->gen_d;
    P.fast_tx0 = x->ftx0;
    P.fast_tz0 = x->ftz0;
    P.fast_tx1 = x->ftx1;
    P.fast_tz1 = x->ftz1;
    P.gen_arith = x->gen_arith;
    P.recs = x->recs_d;
    P.rtile = x->rtile_d;
    P.err = x->err_d;
    P.wav = x->wav;
    P.syn = x->syn;
    P.res = x->res;
    P.ring = x->ring;
    P.strip_len = 2 * x->S * (x->g.nx + x->g.nz);
    P.ring_t0 = 0;
    P.ring_slots = 0x7fffffff;
    P.jump = x->cfg.jump;
    return P;
}

int active_slots(const fwi_ctx* x, int pred_ge)   // shots with nt >= pred_ge
{
    int n = 0;
    while (n < x->nshots && x->nt_slot[n] >= pred_ge) ++n;
    return n;
}

// FWI_SELF_CHECK builds (diagnostics only) synchronise after every launch,
// name the kernel that failed and report the first access that the kernels'
// own checks redirected (g_check: source line, index or address, block).
#ifdef FWI_SELF_CHECK
#define DIAG_SYNC(tag)                                                                                 \
    do {                                                                                               \
        cudaError_t e_ = cudaStreamSynchronize(x->st);                                                \
        if (e_ != cudaSuccess) fprintf(stderr, "FWI diag: %s failed: %s\n", tag, cudaGetErrorString(e_)); \
        CheckRec c_{};                                                                                 \
        if (cudaMemcpyFromSymbol(&c_, g_check, sizeof(c_)) == cudaSuccess && c_.bad) {               \
            fprintf(stderr, "FWI check: %s line %d idx %lld lim %lld blk %d,%d,%d thr %d,%d\n", tag,  \
                    c_.site, c_.idx, c_.lim, c_.bx, c_.by, c_.bz, c_.tx, c_.ty);                       \
            c_ = CheckRec{};                                                                           \
            cudaMemcpyToSymbol(g_check, &c_, sizeof(c_));                                             \
        }                                                                                              \
    } while (0)
#else
#define DIAG_SYNC(tag) do {} while (0)
#endif

RecParams rec_params(const fwi_ctx* x, float* field, int step)
{
    RecParams Q{};
    Q.g = x->g;
    Q.shots = x->shots_d;
    Q.recs = x->samp_d;
    Q.field = field;
    Q.syn = x->syn;
    Q.step = step;
    Q.jump = x->cfg.jump;
    return Q;
}

// The general-tile classes and the receiver sampling run on side streams,
// concurrently with the interior tiles, unless the tuning says serial.
// Self-checking builds keep every launch on st so that DIAG_SYNC sees each
// kernel finish.
bool concurrent(const fwi_ctx* x)
{
#ifdef FWI_SELF_CHECK
    (void)x;
    return false;
#else
    return x->tune.serial == 2;
#endif
}

cudaStream_t class_stream(const fwi_ctx* x, int cls) { return concurrent(x) ? x->side[cls] : x->st; }
// Receiver sampling of step it reads p^{it+1}, which step it+2 overwrites
// first: it runs on its own stream after step it, and step it+2 waits for it.
bool sample_aside(const fwi_ctx* x) { return concurrent(x); }

// Launch order of the general classes (0 = x-general, 1 = z-general, 2 =
// corners).  By default the z-general blocks, the most numerous and longest,
// start first (2.5% shorter forward steps than x, z, corners on the 560 x 1700,
// 64-shot workload).
const int* class_order(const fwi_ctx* x)
{
    static const int z_first[3] = {1, 0, 2}, x_first[3] = {0, 1, 2};
    return x->tune.class_order == 2 ? x_first : z_first;
}

// Grid of a general class of cnt tiles for n shots.  gen_grid 1: one block per
// (tile, shot).  gen_grid k >= 2: k - 1 blocks per SM over the three classes,
// split by the classes' work (tiles x the relative block time measured on the
// 560 x 1700, 64-shot workload: z-general 1, x-general 1.3, corners 2.9), each
// block looping over its class's items, so that the general work would keep
// that many slots on every SM for the whole step instead of running before the
// interior tiles.  Measured slower than gen_grid 1 at every k.
dim3 gen_grid(const fwi_ctx* x, int cls, int cnt, int n)
{
    if (x->tune.gen_grid <= 1) return dim3(cnt, 1, n);
    static const double cost[3] = {1.3, 1.0, 2.9};
    double tot = 0.0;
    for (int c = 0; c < 3; ++c) tot += cost[c] * (x->gen_off[c + 1] - x->gen_off[c]);
    const double share = cost[cls] * cnt / tot;
    const long long want = (long long)std::llround(share * (x->tune.gen_grid - 1) * x->nsm);
    const long long items = (long long)cnt * n;
    return dim3((unsigned)std::max(1LL, std::min(items, want)), 1, 1);
}

// Forks the side streams of the non-empty classes from st.
void fork_classes(fwi_ctx* x)
{
    if (!concurrent(x)) return;
    cudaEventRecord(x->fork_ev, x->st);
    for (int cls = 0; cls < 3; ++cls)
        if (x->gen_off[cls + 1] > x->gen_off[cls]) cudaStreamWaitEvent(x->side[cls], x->fork_ev, 0);
}

// Joins them back: st waits for every class launched since the fork.
void join_classes(fwi_ctx* x)
{
    if (!concurrent(x)) return;
    for (int cls = 0; cls < 3; ++cls)
        if (x->gen_off[cls + 1] > x->gen_off[cls]) {
            cudaEventRecord(x->join_ev[cls], x->side[cls]);
            cudaStreamWaitEvent(x->st, x->join_ev[cls], 0);
        }
}

// The general-tile class cls (0 = x-general, 1 = z-general, 2 = corners) in
// the variant compiled for MB resident blocks per SM.  z-only tiles never
// touch su, srx or the x psi sites, the members of BwdSmem from su on.
template <int MB>
void launch_fwd_gen(int cls, dim3 grid, dim3 block, cudaStream_t cs, const StepParams& P)
{
    if (cls == 0) FWI_LAUNCH((k_fwd_gen<true, false, MB>), grid, block, 0, cs, P);
    if (cls == 1) FWI_LAUNCH((k_fwd_gen<false, true, MB>), grid, block, 0, cs, P);
    if (cls == 2) FWI_LAUNCH((k_fwd_gen<true, true, MB>), grid, block, 0, cs, P);
}
template <int MB>
void launch_bwd_edge(int cls, dim3 grid, dim3 block, cudaStream_t cs, const StepParams& P)
{
    if (cls == 0) FWI_LAUNCH((k_bwd_edge<true, false, MB>), grid, block, sizeof(BwdSmem), cs, P);
    if (cls == 1) FWI_LAUNCH((k_bwd_edge<false, true, MB>), grid, block, offsetof(BwdSmem, su), cs, P);
    if (cls == 2) FWI_LAUNCH((k_bwd_edge<true, true, MB>), grid, block, sizeof(BwdSmem), cs, P);
}
// Dynamic shared memory limits of the backward variants.
template <int MB>
cudaError_t set_bwd_smem()
{
    cudaError_t e = cudaFuncSetAttribute(k_bwd_int<MB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)BWD_INT_SMEM);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_bwd_edge<true, false, MB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(BwdSmem));
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_bwd_edge<false, true, MB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(BwdSmem));
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_bwd_edge<true, true, MB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(BwdSmem));
    return e;
}

// 8th-order steps (fwi_kernels8.cuh): passes over the padded grid of the n
// shots from P.shot_base, on the context's stream.
Step8 step8_buffers(const fwi_ctx* x)
{
    const long long half = (long long)x->nshots * x->g.fstride;
    return Step8{x->X8 + x->origin, x->X8 + half + x->origin, x->X8 + 2 * half + x->origin,
                 x->X8 + 3 * half + x->origin};
}

long long launch_fwd_step8(fwi_ctx* x, StepParams& P, int n)
{
    const dim3 block(32, 8);
    const dim3 gpos((x->g.pnx + 1 + 31) / 32, (x->g.pnz + 1 + 7) / 8, n), gcell((x->g.pnx + 31) / 32, (x->g.pnz + 7) / 8, n);
    const Step8 B = step8_buffers(x);
    FWI_LAUNCH_PDL(k8_uv, gpos, block, 0, x->st, P, B);
    DIAG_SYNC("k8_uv");
    FWI_LAUNCH_PDL(k8_fwd, gcell, block, 0, x->st, P, B);
    DIAG_SYNC("k8_fwd");
    return 2;
}

long long launch_bwd_step8(fwi_ctx* x, StepParams& P, int n)
{
    const dim3 block(32, 8);
    const dim3 gpos((x->g.pnx + 1 + 31) / 32, (x->g.pnz + 1 + 7) / 8, n), gcell((x->g.pnx + 31) / 32, (x->g.pnz + 7) / 8, n);
    const Step8 B = step8_buffers(x);
    long long l = 3;
    FWI_LAUNCH_PDL(k8_adj_uv, gpos, block, 0, x->st, P, B);
    DIAG_SYNC("k8_adj_uv");
    FWI_LAUNCH_PDL(k8_adj, gcell, block, 0, x->st, P, B);
    DIAG_SYNC("k8_adj");
    const int c0 = x->cell8_off[P.shot_base], nc = x->cell8_off[P.shot_base + n] - c0;
    if ((P.step - 1) % x->cfg.jump == 0 && nc > 0) {
        FWI_LAUNCH_PDL(k8_inject, (nc + 127) / 128, 128, 0, x->st, P, x->cells8_d + c0, x->rec8_d, nc,
                   (P.step - 1) / x->cfg.jump);
        DIAG_SYNC("k8_inject");
        ++l;
    }
    FWI_LAUNCH_PDL(k8_rebuild, dim3((x->g.nx + 31) / 32, (x->g.nz + 7) / 8, n), block, 0, x->st, P, B);
    DIAG_SYNC("k8_rebuild");
    return l;
}

// One forward step of the shots [lo, hi): general tiles (one launch per
// class, on the side streams) and interior tiles concurrently, then receiver
// sampling.
long long launch_fwd_step(fwi_ctx* x, StepParams& P, int lo, int hi, bool sample = true)
{
    const dim3 block(BX, BY);
    const int n = hi - lo;
    long long l = 0;
    P.shot_base = lo;
    if (x->samp_pending[P.step & 1]) {                 // the sample of step it-2 read the field this step writes
        cudaStreamWaitEvent(x->st, x->samp_ev[P.step & 1], 0);
        x->samp_pending[P.step & 1] = false;
    }
    if (x->M == 4) {
        l += launch_fwd_step8(x, P, n);
    } else {
    fork_classes(x);
    const int2* gen = P.gen_tiles;
    for (int k = 0; k < 3; ++k) {
        const int cls = class_order(x)[k];
        const int cnt = x->gen_off[cls + 1] - x->gen_off[cls];
        if (!cnt) continue;
        P.gen_tiles = x->gen_d + x->gen_off[cls];
        P.gen_n = cnt;
        P.gen_shots = n;
        const dim3 grid = gen_grid(x, cls, cnt, n);
        cudaStream_t cs = class_stream(x, cls);
        if (x->tune.fwd_gen_blocks == 3) launch_fwd_gen<3>(cls, grid, block, cs, P);
        else launch_fwd_gen<4>(cls, grid, block, cs, P);
        DIAG_SYNC("k_fwd_gen");
        ++l;
    }
    P.gen_tiles = gen;
    if (x->ftx1 > x->ftx0 && x->ftz1 > x->ftz0) {
        const dim3 grid(x->ftx1 - x->ftx0, x->ftz1 - x->ftz0, n);
        if (x->tune.fwd_int_blocks == 4) FWI_LAUNCH(k_fwd_fast<4>, grid, block, 0, x->st, P);
        else FWI_LAUNCH(k_fwd_fast<6>, grid, block, 0, x->st, P);
        DIAG_SYNC("k_fwd_fast");
        ++l;
    }
    join_classes(x);
    }
    if (sample && P.step % x->cfg.jump == 0) {
        RecParams Q = rec_params(x, P.pold, P.step);
        Q.lo = x->samp_off[lo];
        Q.hi = x->samp_off[hi];
        if (Q.hi > Q.lo) {
            cudaStream_t ss = x->st;
            if (sample_aside(x)) {
                cudaEventRecord(x->step_ev, x->st);
                cudaStreamWaitEvent(x->samp_st, x->step_ev, 0);
                ss = x->samp_st;
            }
            FWI_LAUNCH(k_sample, (Q.hi - Q.lo + 255) / 256, 256, 0, ss, Q);
            DIAG_SYNC("k_sample");
            if (sample_aside(x)) {
                cudaEventRecord(x->samp_ev[P.step & 1], x->samp_st);
                x->samp_pending[P.step & 1] = true;
                x->samp_used = true;
            }
            ++l;
        }
    }
    return l;
}

// One backward step of the shots [lo, hi): general tiles (one launch per
// class, on the side streams) and interior tiles concurrently.
long long launch_bwd_step(fwi_ctx* x, StepParams& P, int lo, int hi)
{
    const dim3 block(BX, BY);
    const int n = hi - lo;
    long long l = 0;
    P.shot_base = lo;
    if (x->M == 4) return launch_bwd_step8(x, P, n);
    fork_classes(x);
    // z-only tiles never touch the members of BwdSmem from su on
    const int2* gen = P.gen_tiles;
    for (int k = 0; k < 3; ++k) {
        const int cls = class_order(x)[k];
        const int cnt = x->gen_off[cls + 1] - x->gen_off[cls];
        if (!cnt) continue;
        P.gen_tiles = x->gen_d + x->gen_off[cls];
        P.gen_n = cnt;
        P.gen_shots = n;
        const dim3 grid = gen_grid(x, cls, cnt, n);
        cudaStream_t cs = class_stream(x, cls);
        if ((cls == 1 ? x->tune.bwd_zgen_blocks : x->tune.bwd_gen_blocks) == 3) launch_bwd_edge<3>(cls, grid, block, cs, P);
        else launch_bwd_edge<4>(cls, grid, block, cs, P);
        DIAG_SYNC("k_bwd_edge");
        ++l;
    }
    P.gen_tiles = gen;
    if (x->ftx1 > x->ftx0 && x->ftz1 > x->ftz0) {
        const dim3 grid(x->ftx1 - x->ftx0, x->ftz1 - x->ftz0, n);
        if (x->tune.bwd_int_blocks == 3) FWI_LAUNCH(k_bwd_int<3>, grid, block, BWD_INT_SMEM, x->st, P);
        else FWI_LAUNCH(k_bwd_int<4>, grid, block, BWD_INT_SMEM, x->st, P);
        DIAG_SYNC("k_bwd_int");
        ++l;
    }
    join_classes(x);
    return l;
}

// Field and psi buffers of forward step it (p^it in, p^{it+1} over p^{it-1}).
void set_fwd_ptrs(const fwi_ctx* x, StepParams& P, int it)
{
    const long long half = (long long)x->nshots * x->g.fstride;
    const long long phalf = (long long)x->nshots * x->pl.stride;
    P.step = it;
    P.pcur = x->F + (long long)(it & 1) * half + x->origin;
    P.tm_pcur = x->tm_F[it & 1];
    P.pold = x->F + (long long)((it + 1) & 1) * half + x->origin;
    P.psr = x->psiF + (long long)(it & 1) * phalf;
    P.psw = x->psiF + (long long)((it + 1) & 1) * phalf;
}

// Strip ring of segment j: with strips, every step's strip in its own slot;
// with checkpoints, the strips of p^{t_a - 1} .. p^{t_a + seg} (t_a = j seg)
// in seg + 2 slots.
void set_ring(const fwi_ctx* x, StepParams& P, int j)
{
    if (x->store == FWI_STORE_STRIPS) {
        P.ring_t0 = 0;
        P.ring_slots = 0x7fffffff;
    } else {
        P.ring_t0 = j * x->seg - 2;
        P.ring_slots = x->seg + 2;
    }
}

// Grid of the checkpoint kernels: n shots, each thread both time levels of its cells.
dim3 snap_grid(const fwi_ctx* x, int n)
{
    return dim3((unsigned)std::min<long long>(1024, (x->g.fstride + 255) / 256), 1, (unsigned)n);
}

// Checkpoint of segment j (its start t_a = j seg, taken after forward step
// t_a - 1): p^{t_a} and p^{t_a - 1} (both field halves) and the psi memory
// that step t_a reads, of shots [lo, hi).
long long take_snapshot(fwi_ctx* x, int j, int lo, int hi)
{
    const int n = hi - lo;
    if (n <= 0) return 0;
    const Geo& g = x->g;
    const long long half = (long long)x->nshots * g.fstride, phalf = (long long)x->nshots * x->pl.stride;
    const long long blk = (long long)(j - 1) * x->nshots + lo;            // first (checkpoint, shot) block
    const float* f = x->F + (long long)lo * g.fstride;
    unsigned* amax = x->snapAmax + 2 * blk;
    const dim3 grid = snap_grid(x, n);
    const int ta = j * x->seg, ha = ta & 1;                                // p^{t_a} is in field half ha
    long long l = 0;
    switch (x->cfg.snap_precision) {
    case FWI_SNAP_F32:
        FWI_LAUNCH(k_snap_store<float>, grid, 256, 0, x->st, f, half, g.fstride, ha, nullptr,
                   (float*)x->snapP + blk * 2 * g.fstride);
        l = 1;
        break;
    case FWI_SNAP_F16:
        cudaMemsetAsync(amax, 0, sizeof(unsigned) * 2 * n, x->st);
        FWI_LAUNCH(k_snap_absmax, grid, 256, 0, x->st, f, half, g.fstride, ha, amax);
        FWI_LAUNCH(k_snap_store<__half>, grid, 256, 0, x->st, f, half, g.fstride, ha, amax,
                   (__half*)x->snapP + blk * 2 * g.fstride);
        l = 2;
        break;
    default:
        cudaMemsetAsync(amax, 0, sizeof(unsigned) * 2 * n, x->st);
        FWI_LAUNCH(k_snap_absmax, grid, 256, 0, x->st, f, half, g.fstride, ha, amax);
        FWI_LAUNCH(k_snap_store<__nv_bfloat16>, grid, 256, 0, x->st, f, half, g.fstride, ha, amax,
                   (__nv_bfloat16*)x->snapP + blk * 2 * g.fstride);
        l = 2;
        break;
    }
    cudaMemcpyAsync(x->snapPsi + blk * x->pl.stride, x->psiF + (long long)(ta & 1) * phalf + (long long)lo * x->pl.stride,
                    sizeof(float) * n * x->pl.stride, cudaMemcpyDeviceToDevice, x->st);
    DIAG_SYNC("k_snap_store");
    return l;
}

// Restores the checkpoint of segment j into the forward buffers of shots
// [lo, hi) and writes the strips of the two time levels it holds, p^{t_a - 1}
// and p^{t_a}, into ring slots 0 and 1 (P's ring is that of segment j).
long long restore_snapshot(fwi_ctx* x, StepParams& P, int j, int lo, int hi)
{
    const int n = hi - lo;
    if (n <= 0) return 0;
    const Geo& g = x->g;
    const long long half = (long long)x->nshots * g.fstride, phalf = (long long)x->nshots * x->pl.stride;
    const long long blk = (long long)(j - 1) * x->nshots + lo;
    float* f = x->F + (long long)lo * g.fstride;
    const unsigned* amax = x->snapAmax + 2 * blk;
    const dim3 grid = snap_grid(x, n);
    const int ta = j * x->seg, ha = ta & 1;
    switch (x->cfg.snap_precision) {
    case FWI_SNAP_F32:
        FWI_LAUNCH(k_snap_load<float>, grid, 256, 0, x->st, f, half, g.fstride, ha, nullptr,
                   (const float*)x->snapP + blk * 2 * g.fstride);
        break;
    case FWI_SNAP_F16:
        FWI_LAUNCH(k_snap_load<__half>, grid, 256, 0, x->st, f, half, g.fstride, ha, amax,
                   (const __half*)x->snapP + blk * 2 * g.fstride);
        break;
    default:
        FWI_LAUNCH(k_snap_load<__nv_bfloat16>, grid, 256, 0, x->st, f, half, g.fstride, ha, amax,
                   (const __nv_bfloat16*)x->snapP + blk * 2 * g.fstride);
        break;
    }
    cudaMemcpyAsync(x->psiF + (long long)(ta & 1) * phalf + (long long)lo * x->pl.stride, x->snapPsi + blk * x->pl.stride,
                    sizeof(float) * n * x->pl.stride, cudaMemcpyDeviceToDevice, x->st);
    const dim3 sgrid((P.strip_len + 255) / 256, 1, n);
    P.shot_base = lo;
    for (int lev = 0; lev < 2; ++lev) {                    // p^{t_a - 1}, then p^{t_a}
        const float* f = x->F + (long long)((ta - 1 + lev) & 1) * half + x->origin;
        if (x->S == NSTRIP8) FWI_LAUNCH(k_strips_of_field<NSTRIP8>, sgrid, 256, 0, x->st, P, f, ta - 2 + lev);
        else FWI_LAUNCH(k_strips_of_field<NSTRIP>, sgrid, 256, 0, x->st, P, f, ta - 2 + lev);
    }
    DIAG_SYNC("k_snap_load");
    return 3;
}

// Forward steps [it0, it1) of the shots [lo, hi), each step over those of
// them still active; receiver sampling and checkpoints only in the first
// (full) forward pass.
long long forward_steps(fwi_ctx* x, StepParams& P, int it0, int it1, int lo, int hi, bool first_pass)
{
    long long l = 0;
    for (int it = it0; it < it1; ++it) {
        const int h = std::min(hi, std::max(lo, active_slots(x, it + 1)));
        if (h <= lo) break;
        set_fwd_ptrs(x, P, it);
        l += launch_fwd_step(x, P, lo, h, first_pass);
        if (first_pass && x->store == FWI_STORE_SNAPSHOTS && (it + 1) % x->seg == 0) {
            const int j = (it + 1) / x->seg;
            if (j >= 1 && j <= x->nseg - 2)
                l += take_snapshot(x, j, lo, std::min(hi, std::max(lo, active_slots(x, it + 2))));
        }
    }
    return l;
}

int run_forward(fwi_ctx* x)
{
    const long long half = (long long)x->nshots * x->g.fstride;
    const long long phalf = (long long)x->nshots * x->pl.stride;
    CK(cudaMemsetAsync(x->F, 0, sizeof(float) * 2 * half, x->st));
    CK(cudaMemsetAsync(x->psiF, 0, sizeof(float) * 2 * phalf, x->st));
    StepParams P = base_params(x);
    set_ring(x, P, x->nseg - 1);             // the first pass keeps the strips of the last segment
    long long launches = 0;
    // batched: one launch per step over the active shots; plain: shot after shot
    if (x->cfg.plain_per_shot) {
        for (int grp = 0; grp < x->nshots; ++grp) launches += forward_steps(x, P, 0, x->nt_slot[grp], grp, grp + 1, true);
    } else {
        launches += forward_steps(x, P, 0, x->nt_run, 0, x->nshots, true);
    }
    if (x->samp_used) {                                   // every sample lands before the misfit reads syn
        cudaEventRecord(x->samp_done, x->samp_st);
        cudaStreamWaitEvent(x->st, x->samp_done, 0);
    }
    x->samp_pending[0] = x->samp_pending[1] = false;
    x->samp_used = false;
    CK(cudaGetLastError());
    x->stats.launches = launches;
    return FWI_OK;
}

int run_misfit(fwi_ctx* x)
{
    if (x->msf.kind == FWI_MISFIT_XCORR) {
        // XCORR1D shot by shot (traces of one shot share their length), one sum over all traces
        for (size_t s = 0; s < x->shot_nr.size(); ++s) {
            if (!x->shot_nr[s]) continue;
            const long long o = x->shot_syn_off[s];
            launch_xcorr_traces(x->obs + o, x->syn + o, x->res + o, x->geo_d + x->shot_tr0[s],
                                x->xpart_d + x->shot_tr0[s], x->shot_nr[s], x->shot_nt0[s], x->msf.offset_min,
                                x->msf.offset_max, x->msf.slice, x->st);
            DIAG_SYNC("k_xcorr");
            ++x->stats.launches;
        }
        launch_xcorr_sum(x->xpart_d, x->ntraces, x->mis, x->st);
        DIAG_SYNC("k_xcorr_sum");
        CK(cudaGetLastError());
        x->stats.launches += 1;
        return FWI_OK;
    }
    FWI_LAUNCH(k_misfit, x->npartial, 256, 0, x->st, x->syn, x->obs, x->res, x->nsamples, x->partial);
    DIAG_SYNC("k_misfit");
    FWI_LAUNCH(k_misfit_final, 1, 256, 0, x->st, x->partial, x->npartial, x->mis);
    DIAG_SYNC("k_misfit_final");
    CK(cudaGetLastError());
    x->stats.launches += 2;
    return FWI_OK;
}

// Backward steps m = t_b .. t_a + 1 of shots [lo, hi) (each over those of them
// still active).
long long backward_steps(fwi_ctx* x, StepParams& P, int tb, int ta, int lo, int hi)
{
    const long long half = (long long)x->nshots * x->g.fstride;
    const long long phalf = (long long)x->nshots * x->pl.stride;
    long long l = 0;
    for (int m = tb; m > ta; --m) {
        const int h = std::min(hi, std::max(lo, active_slots(x, m)));
        if (h <= lo) continue;
        P.step = m;
        P.pcur = x->F + (long long)((m - 1) & 1) * half + x->origin;   // p^{m-1}
        P.tm_pcur = x->tm_F[(m - 1) & 1];
        P.pold = x->F + (long long)(m & 1) * half + x->origin;         // p^m -> p^{m-2}
        P.bcur = x->A + (long long)((m + 1) & 1) * half + x->origin;   // b^{m+1}
        P.tm_bcur = x->tm_A[(m + 1) & 1];
        P.bold = x->A + (long long)(m & 1) * half + x->origin;         // b^{m+2} -> b^m
        P.psr = x->psiA + (long long)(m & 1) * phalf;
        P.psw = x->psiA + (long long)((m + 1) & 1) * phalf;
        l += launch_bwd_step(x, P, lo, h);
    }
    return l;
}

// The backward half of shots [lo, hi) whose longest record is nt_grp steps,
// segment by segment, last first.  With strips there is one segment and the
// forward pass left everything it needs.  With checkpoints, every segment
// but the last (whose strips the forward pass kept) is first recomputed from
// its checkpoint (segment 0 from rest), its strips going to the ring.
long long backward_segments(fwi_ctx* x, StepParams& P, int nt_grp, int lo, int hi)
{
    const long long half = (long long)x->nshots * x->g.fstride;
    const long long phalf = (long long)x->nshots * x->pl.stride;
    const int seg = x->seg;
    const int nseg_grp = (nt_grp + seg - 1) / seg;
    long long l = 0;
    for (int j = nseg_grp - 1; j >= 0; --j) {
        const int ta = j * seg, tb = std::min(ta + seg, nt_grp);
        set_ring(x, P, j);
        if (x->store == FWI_STORE_SNAPSHOTS && j < x->nseg - 1) {
            const int h = std::min(hi, std::max(lo, active_slots(x, ta + 1)));
            if (h <= lo) continue;
            if (j == 0) {
                for (int k = 0; k < 2; ++k) {
                    cudaMemsetAsync(x->F + k * half + (long long)lo * x->g.fstride, 0,
                                    sizeof(float) * (h - lo) * x->g.fstride, x->st);
                    cudaMemsetAsync(x->psiF + k * phalf + (long long)lo * x->pl.stride, 0,
                                    sizeof(float) * (h - lo) * x->pl.stride, x->st);
                }
            } else {
                l += restore_snapshot(x, P, j, lo, h);
            }
            l += forward_steps(x, P, ta, tb, lo, h, false);
        }
        l += backward_steps(x, P, tb, ta, lo, hi);
    }
    return l;
}

int run_backward(fwi_ctx* x)
{
    const long long half = (long long)x->nshots * x->g.fstride;
    const long long phalf = (long long)x->nshots * x->pl.stride;
    CK(cudaMemsetAsync(x->A, 0, sizeof(float) * 2 * half, x->st));
    CK(cudaMemsetAsync(x->psiA, 0, sizeof(float) * 2 * phalf, x->st));
    CK(cudaMemsetAsync(x->Gacc, 0, sizeof(float) * half, x->st));
    StepParams P = base_params(x);
    P.gacc = x->Gacc + x->origin;
    long long launches = 0;
    if (x->cfg.plain_per_shot) {
        for (int grp = 0; grp < x->nshots; ++grp) launches += backward_segments(x, P, x->nt_slot[grp], grp, grp + 1);
    } else {
        launches += backward_segments(x, P, x->nt_run, 0, x->nshots);
    }
    CK(cudaGetLastError());
    // FP64 reduction over shots and the 2/v factor
    FWI_LAUNCH(k_reduce, dim3((x->g.nx + 255) / 256, x->g.nz), 256, 0, x->st, x->Gacc + x->origin, x->vel, x->grad, x->g, x->nshots);
    CK(cudaGetLastError());
    x->stats.launches += launches + 1;
    return FWI_OK;
}

float event_ms(cudaEvent_t a, cudaEvent_t b)
{
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, a, b) != cudaSuccess) { cudaGetLastError(); return 0.f; }
    return ms;
}

// A block whose tile copy did not land within its bounded wait skipped its
// tile and returned; the fields it should have written, and every later step,
// are undefined.  The context then refuses further work (usable()).
int finish(fwi_ctx* x)
{
    CK(cudaStreamSynchronize(x->st));
    int bad = 0;
    CK(cudaMemcpy(&bad, x->err_d, sizeof(int), cudaMemcpyDeviceToHost));
    if (bad) {
        x->broken = true;
        x->have_fwd = false;
        return fail(x, FWI_ERR_CUDA, "a tile copy (TMA) did not complete within its bounded wait; the results are "
                                     "undefined and the context refuses further work: destroy and recreate it");
    }
    return FWI_OK;
}

int usable(fwi_ctx* x)
{
    if (x->broken)
        return fail(x, FWI_ERR_STATE, "a tile copy timed out earlier: destroy and recreate the context");
    return FWI_OK;
}

// The TMA map of one field half (base: its first float): dims (ld, rows,
// slots) of floats with the fields' strides, box SPW x SPH x 1, no swizzle,
// zero fill outside.  cuTensorMapEncodeTiled comes through the runtime's
// driver entry point, so the library links no driver library.
int encode_field_map(TensorMap* out, float* base, const Geo& g, int rows, int slots)
{
#ifdef FWI_CPU_EMU
    (void)base; (void)g; (void)rows; (void)slots;
    *out = TensorMap{};
    return 0;
#else
    static PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
    if (!encode) {
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess || !f)
            return -1;
        encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(f);
    }
    static_assert(sizeof(CUtensorMap) == sizeof(TensorMap), "a TensorMap holds one CUtensorMap");
    CUtensorMap m;
    const cuuint64_t dims[3] = {(cuuint64_t)g.ld, (cuuint64_t)rows, (cuuint64_t)slots};
    const cuuint64_t strides[2] = {(cuuint64_t)g.ld * sizeof(float), (cuuint64_t)g.fstride * sizeof(float)};
    const cuuint32_t box[3] = {(cuuint32_t)SPW, (cuuint32_t)SPH, 1};
    const cuuint32_t unit[3] = {1, 1, 1};
    if (encode(&m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, base, dims, strides, box, unit, CU_TENSOR_MAP_INTERLEAVE_NONE,
               CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) !=
        CUDA_SUCCESS)
        return -1;
    std::memcpy(out, &m, sizeof m);
    return 0;
#endif
}

enum Phase { PH_FWD = 0, PH_MIS = 1, PH_BWD = 2 };

int run_phase_direct(fwi_ctx* x, int ph)
{
    return ph == PH_FWD ? run_forward(x) : ph == PH_MIS ? run_misfit(x) : run_backward(x);
}

// Runs one phase between its two timing events (forward ev0/ev1, misfit
// ev4/ev5, backward ev2/ev3).  With use_graph the phase is captured once
// into a CUDA graph and replayed; the events stay outside the graphs so that
// their elapsed times are defined.
int run_phase(fwi_ctx* x, int ph, bool graph)
{
    static const int evs[3][2] = {{0, 1}, {4, 5}, {2, 3}};
    CK(cudaEventRecord(x->ev[evs[ph][0]], x->st));
    if (!graph) {
        int s = run_phase_direct(x, ph);
        if (s) return s;
    } else {
        if (!x->gexec[ph]) {
            const long long before = x->stats.launches;
            CK(cudaStreamBeginCapture(x->st, cudaStreamCaptureModeThreadLocal));
            int s = run_phase_direct(x, ph);
            cudaGraph_t gr = nullptr;
            cudaError_t e = cudaStreamEndCapture(x->st, &gr);
            if (s) { if (gr) cudaGraphDestroy(gr); return s; }
            if (e != cudaSuccess) return cuda_fail(x, e, "cudaStreamEndCapture");
            x->graph[ph] = gr;
            e = cudaGraphInstantiate(&x->gexec[ph], gr, 0);
            if (e != cudaSuccess) { drop_graph(x); return cuda_fail(x, e, "cudaGraphInstantiate"); }
            x->graph_launches[ph] = ph == PH_FWD ? x->stats.launches : x->stats.launches - before;
        }
        CK(cudaGraphLaunch(x->gexec[ph], x->st));
    }
    CK(cudaEventRecord(x->ev[evs[ph][1]], x->st));
    return FWI_OK;
}

// Device bytes of the forward-field storage with nseg segments of
// ceil(nt_run / nseg) steps: nseg - 2 checkpoints (two pressure fields in the
// storage type, the psi memory and two scale words per shot) and a ring of
// seg + 2 strip slots per shot.
long long snapshot_bytes(const fwi_ctx* x, int nshots, int nt_run, int nseg)
{
    const long long seg = (nt_run + nseg - 1) / nseg;
    const long long nseg_eff = (nt_run + seg - 1) / seg;
    const long long elem = x->cfg.snap_precision == FWI_SNAP_F32 ? 4 : 2;
    const long long per_ckpt = (long long)nshots * (2 * x->g.fstride * elem + 4 * x->pl.stride + 8);
    const long long strip_b = 2LL * x->S * (x->g.nx + x->g.nz) * 4;
    return std::max(0LL, nseg_eff - 2) * per_ckpt + (seg + 2) * nshots * strip_b;
}

// Picks the forward-field storage of a shot set (cfg.store, FWI_STORE_AUTO:
// the strip ring when the whole shot state fits the budget, else the segment
// count with the least memory) and sets store, seg, nseg and nsnap.
int choose_store(fwi_ctx* x, int nshots, int nt_run, long long base_b, long long strips_b)
{
    int mode = x->cfg.store;
    int nseg = x->cfg.snapshots;
    if (mode == FWI_STORE_AUTO) {
        long long budget = (long long)x->cfg.hbm_budget_mb << 20;
        if (!budget) {
            size_t fr = 0, tot = 0;
            if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) { cudaGetLastError(); fr = 0; }
            budget = (long long)(0.9 * (double)fr);
        }
        if (base_b + strips_b <= budget) {
            mode = FWI_STORE_STRIPS;
        } else {
            long long best = -1;
            for (int n = 1; n <= nt_run; ++n) {
                const long long b = snapshot_bytes(x, nshots, nt_run, n);
                if (best < 0 || b < best) { best = b; nseg = n; }
                if (n > 4 && b > 2 * best) break;            // past the minimum: memory grows with n
            }
            if (base_b + best > budget)
                return fail(x, FWI_ERR_NOMEM, "the shot state needs " + std::to_string((base_b + best) >> 20) +
                                                  " MiB even with checkpoints; the budget is " +
                                                  std::to_string(budget >> 20) + " MiB");
            mode = FWI_STORE_SNAPSHOTS;
        }
    } else if (mode == FWI_STORE_SNAPSHOTS && nseg == 0) {
        nseg = (int)std::ceil(std::sqrt((double)nt_run));
    }
    if (mode == FWI_STORE_STRIPS) {
        x->store = FWI_STORE_STRIPS;
        x->seg = nt_run;
        x->nseg = 1;
        x->nsnap = 0;
        return FWI_OK;
    }
    nseg = std::max(1, std::min(nseg, nt_run));
    x->store = FWI_STORE_SNAPSHOTS;
    x->seg = (nt_run + nseg - 1) / nseg;
    x->nseg = (nt_run + x->seg - 1) / x->seg;
    x->nsnap = std::max(0, x->nseg - 2);
    return FWI_OK;
}

// Defaults of fwi_tuning: the interior tile rectangle starts at the first
// column (row) whose stencils reach no edge, CPML or strip cell.
fwi_tuning default_tuning(const fwi_ctx* x)
{
    fwi_tuning t{};
    const int np = x->cfg.npml;
    t.x_first = (int)round_up(std::max(8, np + 5), 4);
    t.z_first = x->cfg.free_surface ? 8 : (int)round_up(std::max(8, np + 5), R);
    t.fwd_gen_blocks = 4;
    t.bwd_gen_blocks = 3;           // 80 registers: the psi-site tables made the 64-register variant 11% slower
    t.bwd_zgen_blocks = 4;          // the z-general class alone: 1% faster per backward step at 4 (C2 grid)
    t.fwd_int_blocks = 6;
    t.bwd_int_blocks = 4;
    t.class_order = 1;
    t.serial = 2;
    t.priority = 1;
    t.gen_grid = 1;
    return t;
}

// (Re)creates the general classes' side streams at the tuning's priority.
cudaError_t make_side_streams(fwi_ctx* x)
{
    int least = 0, greatest = 0;
    cudaError_t e = cudaDeviceGetStreamPriorityRange(&least, &greatest);
    if (e != cudaSuccess) return e;
    for (int i = 0; i < 3; ++i) {
        if (x->side[i]) cudaStreamDestroy(x->side[i]);
        x->side[i] = nullptr;
        e = cudaStreamCreateWithPriority(&x->side[i], cudaStreamNonBlocking, x->tune.priority == 2 ? greatest : 0);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

// Tile grid and field layout of the padded grid (tuning x_first, z_first),
// the interior tile rectangle, the general tile list, and K in that layout
// (zero; fwi_set_model fills it).
int set_layout(fwi_ctx* x)
{
    if (x->gen_d) { cudaFree(x->gen_d); x->bytes_model -= sizeof(int2) * (size_t)std::max(1, x->ngen); x->gen_d = nullptr; }
    if (x->K) { cudaFree(x->K); x->bytes_model -= sizeof(float) * (size_t)x->g.fstride; x->K = nullptr; }
    const fwi_config* cfg = &x->cfg;
    Geo& g = x->g;
    g.nx = cfg->nx; g.nz = cfg->nz; g.npml = cfg->npml; g.fs = cfg->free_surface;
    g.pnx = cfg->nx + 2 * cfg->npml;                         // fwi_2d.c:155
    g.pnz = cfg->nz + (g.fs ? 1 : 2) * cfg->npml;            // fwi_2d.c:155,162
    g.x0p = cfg->npml; g.z0p = g.fs ? 0 : cfg->npml;
    // Tile grid in x: the first interior tile starts at the first column x0i
    // (a multiple of 4, for 16-byte staging) whose stencils reach no edge,
    // CPML or strip cell; tile column 0 starts xoff <= 0 columns earlier.
    // The left zero margin mx covers the halo of that first tile, and makes
    // every tile's staged rows start on a 128-byte boundary.
    const int x0i = x->tune.x_first;
    g.xoff = x0i - TX * ((x0i + TX - 1) / TX);
    const int mx = HX - g.xoff;                              // (mx + xoff - HX) == 0: aligned rows
    g.ntx = (g.pnx - g.xoff + TX - 1) / TX;
    // The same in z: the first interior tile starts at row z0i (a multiple
    // of R, so the warp holding row 0 starts there, as the top formulas
    // assume) and tile row 0 starts zoff <= 0 rows earlier, above a margin
    // of MZ zero rows.
    const int z0i = x->tune.z_first;
    g.zoff = z0i - TZ * ((z0i + TZ - 1) / TZ);
    const int mz = MZ - g.zoff;
    g.ntz = (g.pnz - g.zoff + TZ - 1) / TZ;
    g.ld = (int)round_up(mx + g.xoff + (long long)g.ntx * TX + HX, 32);
    x->rows_alloc = mz + g.zoff + g.ntz * TZ + MZ;
    g.fstride = (long long)x->rows_alloc * g.ld;
    x->origin = (long long)mz * g.ld + mx;

    // interior tile rectangle and the list of general-path tiles
    {
        std::vector<int2> gen;
        int tx0 = -1, tx1 = -1, tz0 = -1, tz1 = -1;
        for (int t = 0; t < g.ntx; ++t)
            if (!tile_x_general(g, g.xoff + t * TX)) { if (tx0 < 0) tx0 = t; tx1 = t + 1; }
        for (int t = 0; t < g.ntz; ++t)
            if (!tile_z_general(g, g.zoff + t * TZ)) { if (tz0 < 0) tz0 = t; tz1 = t + 1; }
        if (tx0 < 0 || tz0 < 0) tx0 = tx1 = tz0 = tz1 = 0;
        // general tiles grouped by class: 0 = x-general only, 1 = z-general only, 2 = both
        for (int cls = 0; cls < 3; ++cls) {
            x->gen_off[cls] = (int)gen.size();
            for (int tz = 0; tz < g.ntz; ++tz)
                for (int tx = 0; tx < g.ntx; ++tx) {
                    if (tx >= tx0 && tx < tx1 && tz >= tz0 && tz < tz1) continue;
                    const bool gx = tile_x_general(g, g.xoff + tx * TX), gz = tile_z_general(g, g.zoff + tz * TZ);
                    if (!gx && !gz) return fail(x, FWI_ERR_ARG, "tile classes do not form a rectangle");
                    if ((gx && !gz && cls == 0) || (!gx && gz && cls == 1) || (gx && gz && cls == 2))
                        gen.push_back(make_int2(tx, tz));
                }
        }
        x->gen_off[3] = (int)gen.size();
        x->gen_arith = 1;                                   // the kernels may compute the tiles instead
        for (int cls = 0; cls < 3; ++cls)
            for (int i = x->gen_off[cls]; i < x->gen_off[cls + 1]; ++i) {
                const int2 a = gen_tile_at(g, tx0, tx1, tz0, tz1, cls != 1, cls != 0, i - x->gen_off[cls]);
                if (a.x != gen[i].x || a.y != gen[i].y) x->gen_arith = 0;
            }
        x->ftx0 = tx0; x->ftx1 = tx1; x->ftz0 = tz0; x->ftz1 = tz1;
        x->ngen = (int)gen.size();
        if (int e = dalloc(x, &x->gen_d, gen.size(), &x->bytes_model)) return e;
        if (!gen.empty() && cudaMemcpy(x->gen_d, gen.data(), gen.size() * sizeof(int2), cudaMemcpyHostToDevice) != cudaSuccess)
            return fail(x, FWI_ERR_CUDA, "upload of the general tile list failed");
    }

    if (int e = dalloc(x, &x->K, (size_t)g.fstride, &x->bytes_model)) return e;
    // on the context's stream: a legacy-stream memset would not be ordered
    // before k_build_K, which runs on the non-blocking stream
    if (cudaMemsetAsync(x->K, 0, sizeof(float) * g.fstride, x->st) != cudaSuccess ||
        cudaStreamSynchronize(x->st) != cudaSuccess)
        return fail(x, FWI_ERR_CUDA, "clearing K failed");
    return FWI_OK;
}

// Traces longer than the XCORR kernel's shared memory holds?
bool xcorr_too_long(const fwi_ctx* x)
{
    for (int nt0 : x->shot_nt0)
        if (xcorr_smem_bytes(nt0) > XCORR_MAX_SMEM) return true;
    return false;
}

}  // namespace

extern "C" {

int fwi_version(void) { return kVersion; }

const char* fwi_status_string(int s)
{
    switch (s) {
    case FWI_OK: return "ok";
    case FWI_ERR_ARG: return "invalid argument";
    case FWI_ERR_GEOMETRY: return "source or receiver outside the model";
    case FWI_ERR_NOMEM: return "out of memory";
    case FWI_ERR_CUDA: return "CUDA error";
    case FWI_ERR_STATE: return "call out of order";
    case FWI_ERR_CFL: return "model violates the CFL limit";
    case FWI_ERR_NONFINITE: return "non-finite input";
    case FWI_ERR_NODEVICE: return "no usable sm_103 device";
    default: return "unknown status";
    }
}

const char* fwi_last_error(const fwi_ctx* x) { return x ? x->err.c_str() : "null context"; }

int fwi_cpml_profile(int npml, float d, float dt, float max_f, float max_v, float coef_r, float* a, float* b)
{
    if (npml < 1 || !(d > 0) || !(dt > 0) || !a || !b) return FWI_ERR_ARG;
    cpml_profile(a, b, npml, d, dt, max_f, max_v, coef_r);
    return FWI_OK;
}

int fwi_fd_coefficients(float dx, float dz, float* out8)
{
    if (!(dx > 0) || !(dz > 0) || !out8) return FWI_ERR_ARG;
    fd_coefficients(dx, dz, out8);
    return FWI_OK;
}

int fwi_cell_of(float x, float z, float dx, float dz, int* ix, int* iz)
{
    if (!(dx > 0) || !(dz > 0) || !ix || !iz) return FWI_ERR_ARG;
    cell_of(x, z, dx, dz, ix, iz);
    return FWI_OK;
}

int fwi_check_config(const fwi_config* cfg)
{
    if (!cfg) return FWI_ERR_ARG;
    if (cfg->nx < 8 || cfg->nz < 8 || cfg->npml < 1 || cfg->npml > 256) return FWI_ERR_ARG;
    if (!(cfg->dx > 0) || !(cfg->dz > 0) || !(cfg->dt > 0)) return FWI_ERR_ARG;
    if (cfg->nt_max < 1 || cfg->jump < 1) return FWI_ERR_ARG;
    if (!(cfg->pml_max_f > 0) || !(cfg->pml_max_v > 0) || !(cfg->pml_coef_r > 0 && cfg->pml_coef_r < 1)) return FWI_ERR_ARG;
    if (cfg->free_surface != 0 && cfg->free_surface != 1) return FWI_ERR_ARG;
    if ((cfg->use_graph != 0 && cfg->use_graph != 1) || (cfg->plain_per_shot != 0 && cfg->plain_per_shot != 1))
        return FWI_ERR_ARG;
    if (cfg->store < FWI_STORE_AUTO || cfg->store > FWI_STORE_SNAPSHOTS || cfg->snapshots < 0 ||
        cfg->snap_precision < FWI_SNAP_F32 || cfg->snap_precision > FWI_SNAP_BF16 || cfg->hbm_budget_mb < 0)
        return FWI_ERR_ARG;
    if (cfg->fd_order != 0 && cfg->fd_order != 4 && cfg->fd_order != 8) return FWI_ERR_ARG;
    if (cfg->reserved[0]) return FWI_ERR_ARG;
    return FWI_OK;
}

fwi_ctx* fwi_create(const fwi_config* cfg, int* status)
{
    int st = fwi_check_config(cfg);
    if (st) { if (status) *status = st; return nullptr; }
    fwi_ctx* x = new (std::nothrow) fwi_ctx();
    if (!x) { if (status) *status = FWI_ERR_NOMEM; return nullptr; }
    x->cfg = *cfg;
    auto bail = [&](int code) -> fwi_ctx* {
        if (status) *status = code;
        fwi_destroy(x);
        return nullptr;
    };
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || cfg->device < 0 || cfg->device >= ndev) {
        cudaGetLastError();
        return bail(FWI_ERR_NODEVICE);
    }
    cudaDeviceProp prop{};
    if (cudaGetDeviceProperties(&prop, cfg->device) != cudaSuccess || prop.major != 10 || prop.minor != 3) {
        cudaGetLastError();
        return bail(FWI_ERR_NODEVICE);
    }
    if (cudaSetDevice(cfg->device) != cudaSuccess) return bail(FWI_ERR_NODEVICE);
    if (cudaDeviceGetAttribute(&x->nsm, cudaDevAttrMultiProcessorCount, cfg->device) != cudaSuccess || x->nsm < 1)
        return bail(FWI_ERR_CUDA);
    if (cudaStreamCreateWithFlags(&x->own, cudaStreamNonBlocking) != cudaSuccess) return bail(FWI_ERR_CUDA);
    x->st = x->own;
    for (auto& e : x->ev)
        if (cudaEventCreate(&e) != cudaSuccess) return bail(FWI_ERR_CUDA);
    x->tune = default_tuning(x);
#ifdef FWI_TIMELINE
    if (const char* st = std::getenv("FWI_TIMELINE_STEP")) {
        const char* out = std::getenv("FWI_TIMELINE_OUT");
        x->tl_out = out ? out : "timeline.bin";
        const size_t bytes = sizeof(unsigned long long) * 8 * TL_ITEMS * 2;
        const int step = std::atoi(st);
        if (cudaMalloc(&x->tl_d, bytes) != cudaSuccess || cudaMemset(x->tl_d, 0, bytes) != cudaSuccess ||
            cudaMemcpyToSymbol(g_tl, &x->tl_d, sizeof(x->tl_d)) != cudaSuccess ||
            cudaMemcpyToSymbol(g_tl_step, &step, sizeof(int)) != cudaSuccess)
            return bail(FWI_ERR_CUDA);
    }
#endif
    if (make_side_streams(x) != cudaSuccess) return bail(FWI_ERR_CUDA);
    for (int i = 0; i < 3; ++i)
        if (cudaEventCreateWithFlags(&x->join_ev[i], cudaEventDisableTiming) != cudaSuccess) return bail(FWI_ERR_CUDA);
    if (cudaEventCreateWithFlags(&x->fork_ev, cudaEventDisableTiming) != cudaSuccess) return bail(FWI_ERR_CUDA);
    if (cudaStreamCreateWithFlags(&x->samp_st, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&x->step_ev, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&x->samp_ev[0], cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&x->samp_ev[1], cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&x->samp_done, cudaEventDisableTiming) != cudaSuccess ||
        cudaStreamCreateWithFlags(&x->obs_st, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&x->obs_ev, cudaEventDisableTiming) != cudaSuccess)
        return bail(FWI_ERR_CUDA);

    if (int st = set_layout(x)) return bail(st);
    if (dalloc(x, &x->err_d, 1, &x->bytes_model) || cudaMemset(x->err_d, 0, sizeof(int)) != cudaSuccess)
        return bail(FWI_ERR_NOMEM);
    Geo& g = x->g;

    float fd[8];
    fd_coefficients(cfg->dx, cfg->dz, fd);
    Coef& c = x->c;
    c.c0x = fd[0]; c.c1x = fd[1]; c.ix = fd[2]; c.c0z = fd[3]; c.c1z = fd[4]; c.iz = fd[5];
    c.iz840 = fd[6]; c.iz24 = fd[7];
    c.iarea = 1.0 / (cfg->dx * cfg->dz);                    // fwi_2d.c:216
    x->M = cfg->fd_order == 8 ? 4 : 2;
    x->S = 2 * x->M - 1;
    {   // 8th-order staggered weights / h, w_k / h rounded to float
        static const double w[4] = {1225.0 / 1024.0, -245.0 / 3072.0, 49.0 / 5120.0, -5.0 / 7168.0};
        for (int k = 0; k < 4; ++k) {
            c.w8x[k] = (float)(w[k] / (double)cfg->dx);
            c.w8z[k] = (float)(w[k] / (double)cfg->dz);
        }
    }
    {   // D- D+ along x in one symmetric 7-point stencil (interior tiles)
        const double a = c.c0x, b = c.c1x;
        c.wx1 = (float)(a * a - 2.0 * a * b);
        c.wx2 = (float)(2.0 * a * b);
        c.wx3 = (float)(b * b);
    }

    const int np = cfg->npml, n2 = 2 * np + 1;
    PsiLayout& pl = x->pl;
    long long off = 0;
    pl.u0 = (int)off;  off += (long long)g.pnz * (np + 1);
    pl.u1 = (int)off;  off += (long long)g.pnz * (np + 1);
    pl.v0 = (int)off;  off += (long long)(np + 1) * g.pnx;
    pl.v1 = (int)off;  off += (long long)(np + 1) * g.pnx;
    pl.ux0 = (int)off; off += (long long)g.pnz * np;
    pl.ux1 = (int)off; off += (long long)g.pnz * np;
    pl.vz0 = (int)off; off += (long long)np * g.pnx;
    pl.vz1 = (int)off; off += (long long)np * g.pnx;
    pl.stride = round_up(off, 32);

    // CPML profiles: a0/b0 from cpml_coe, a1/b1 mirrored (fwi_2d.c:272-283)
    std::vector<float> h(8 * n2);
    float *a0x = &h[0], *b0x = &h[n2], *a1x = &h[2 * n2], *b1x = &h[3 * n2];
    float *a0z = &h[4 * n2], *b0z = &h[5 * n2], *a1z = &h[6 * n2], *b1z = &h[7 * n2];
    cpml_profile(a0x, b0x, np, cfg->dx, cfg->dt, cfg->pml_max_f, cfg->pml_max_v, cfg->pml_coef_r);
    cpml_profile(a0z, b0z, np, cfg->dz, cfg->dt, cfg->pml_max_f, cfg->pml_max_v, cfg->pml_coef_r);
    for (int i = 0; i < n2; ++i) {
        a1x[i] = a0x[2 * np - i]; b1x[i] = b0x[2 * np - i];
        a1z[i] = a0z[2 * np - i]; b1z[i] = b0z[2 * np - i];
    }
    if (dalloc(x, &x->pmlc, h.size(), &x->bytes_model)) return bail(FWI_ERR_NOMEM);
    if (dalloc(x, &x->vel, (size_t)g.nx * g.nz, &x->bytes_model)) return bail(FWI_ERR_NOMEM);
    if (dalloc(x, &x->grad, (size_t)g.nx * g.nz, &x->bytes_model)) return bail(FWI_ERR_NOMEM);
    if (dalloc(x, &x->gradf, (size_t)g.nx * g.nz, &x->bytes_model)) return bail(FWI_ERR_NOMEM);
    if (cudaMemcpy(x->pmlc, h.data(), h.size() * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess) return bail(FWI_ERR_CUDA);
    if (set_bwd_smem<3>() != cudaSuccess || set_bwd_smem<4>() != cudaSuccess) return bail(FWI_ERR_CUDA);
    if (status) *status = FWI_OK;
    return x;
}

void fwi_destroy(fwi_ctx* x)
{
    if (!x) return;
#ifdef FWI_TIMELINE
    if (x->tl_d) {
        std::vector<unsigned long long> h((size_t)8 * TL_ITEMS * 2);
        if (cudaMemcpy(h.data(), x->tl_d, h.size() * sizeof(h[0]), cudaMemcpyDeviceToHost) == cudaSuccess) {
            if (FILE* f = std::fopen(x->tl_out.c_str(), "wb")) {
                std::fwrite(h.data(), sizeof(h[0]), h.size(), f);
                std::fclose(f);
            }
        }
        unsigned long long* none = nullptr;
        cudaMemcpyToSymbol(g_tl, &none, sizeof(none));
        cudaFree(x->tl_d);
    }
#endif
    free_shots(x);
    void* ps[] = {x->K, x->vel, x->pmlc, x->grad, x->gradf, x->gen_d, x->err_d};
    for (void* p : ps) if (p) cudaFree(p);
    for (auto& e : x->ev) if (e) cudaEventDestroy(e);
    for (auto& e : x->join_ev) if (e) cudaEventDestroy(e);
    if (x->fork_ev) cudaEventDestroy(x->fork_ev);
    for (cudaEvent_t e : {x->step_ev, x->samp_ev[0], x->samp_ev[1], x->samp_done, x->obs_ev}) if (e) cudaEventDestroy(e);
    for (cudaStream_t t : {x->samp_st, x->obs_st}) if (t) cudaStreamDestroy(t);
    for (auto& t : x->side) if (t) cudaStreamDestroy(t);
    if (x->own) cudaStreamDestroy(x->own);
    delete x;
}

int fwi_set_model(fwi_ctx* x, const float* vel)
{
    if (!x || !vel) return fail(x, FWI_ERR_ARG, "null argument");
    const Geo& g = x->g;
    const size_t n = (size_t)g.nx * g.nz;
    float vmax = 0.f;
    for (size_t i = 0; i < n; ++i) {
        const float v = vel[i];
        if (!std::isfinite(v)) return fail(x, FWI_ERR_NONFINITE, "non-finite velocity at index " + std::to_string(i));
        if (!(v > 0.f)) return fail(x, FWI_ERR_ARG, "non-positive velocity at index " + std::to_string(i));
        vmax = std::max(vmax, v);
    }
    // leapfrog stability of the staggered pair: v dt sum|w_k| sqrt(1/dx^2+1/dz^2) <= 1, with the
    // 4th-order pair (fwi_2d.c:307-311) or the 8th-order weights
    const double wsum = x->M == 4 ? 1225.0 / 1024.0 + 245.0 / 3072.0 + 49.0 / 5120.0 + 5.0 / 7168.0
                                  : 1.129042 + 0.04301412;
    const double cfl = (double)vmax * x->cfg.dt * wsum *
                       std::sqrt(1.0 / ((double)x->cfg.dx * x->cfg.dx) + 1.0 / ((double)x->cfg.dz * x->cfg.dz));
    if (cfl > 1.0) return fail(x, FWI_ERR_CFL, "CFL number " + std::to_string(cfl) + " > 1");
    CK(cudaSetDevice(x->cfg.device));
    CK(cudaMemcpyAsync(x->vel, vel, n * sizeof(float), cudaMemcpyHostToDevice, x->st));
    FWI_LAUNCH(k_build_K, dim3((g.pnx + 255) / 256, g.pnz), 256, 0, x->st, x->vel, x->K + x->origin, g, x->cfg.dt);
    CK(cudaGetLastError());
    int s = finish(x);
    if (s) return s;
    x->have_model = true;
    x->have_fwd = false;
    return FWI_OK;
}

int fwi_set_shots(fwi_ctx* x, int nshots, const fwi_shot* shots)
{
    if (!x || nshots < 1 || !shots) return fail(x, FWI_ERR_ARG, "need at least one shot");
    if (nshots > MAX_SHOTS) return fail(x, FWI_ERR_ARG, "at most " + std::to_string(MAX_SHOTS) + " shots per batch");
    CK(cudaSetDevice(x->cfg.device));
    const Geo& g = x->g;
    const int jump = x->cfg.jump;
    // validate and convert geometry (fwi_2d.c:357-371)
    std::vector<ShotDev> sd(nshots);
    struct Rec { long long foff, syn_base; };
    std::vector<std::vector<Rec>> recs(nshots);
    long long syn_off = 0, wav_tot = 0;
    std::vector<long long> wav_off(nshots);
    std::vector<long long> tr_syn_off(nshots);
    std::vector<int> tr0(nshots), tr_nr(nshots), tr_nt0(nshots);
    std::vector<float4> geo;                      // per trace, input order (XCORR offsets)
    for (int s = 0; s < nshots; ++s) {
        const fwi_shot& sh = shots[s];
        if (sh.nt < 1 || sh.nt > x->cfg.nt_max || (sh.nt - 1) % jump != 0)
            return fail(x, FWI_ERR_ARG, "shot " + std::to_string(s) + ": nt must be in [1, nt_max] with (nt-1) % jump == 0");
        if (sh.nr < 0 || (sh.nr > 0 && !sh.rec_xz) || !sh.wavelet)
            return fail(x, FWI_ERR_ARG, "shot " + std::to_string(s) + ": missing receivers or wavelet");
        int ix, iz;
        cell_of(sh.src_x, sh.src_z, x->cfg.dx, x->cfg.dz, &ix, &iz);
        if (ix < 0 || ix >= g.nx || iz < 0 || iz >= g.nz)
            return fail(x, FWI_ERR_GEOMETRY, "shot " + std::to_string(s) + ": source outside the model");
        for (int i = 0; i < sh.nt; ++i)
            if (!std::isfinite(sh.wavelet[i])) return fail(x, FWI_ERR_NONFINITE, "non-finite wavelet sample");
        if (wav_tot + sh.nt > INT_MAX) return fail(x, FWI_ERR_ARG, "more than 2^31 - 1 wavelet samples in the batch");
        ShotDev& d = sd[s];
        d.nt = sh.nt; d.nt0 = (sh.nt - 1) / jump + 1; d.nr = sh.nr;
        d.src_r = iz + g.z0p; d.src_c = ix + g.x0p;
        d.syn_off = syn_off;
        wav_off[s] = wav_tot;
        d.wav_off = (int)wav_tot;
        wav_tot += sh.nt;
        recs[s].resize(sh.nr);
        for (int r = 0; r < sh.nr; ++r) {
            int rx, rz;
            cell_of(sh.rec_xz[2 * r], sh.rec_xz[2 * r + 1], x->cfg.dx, x->cfg.dz, &rx, &rz);
            if (rx < 0 || rx >= g.nx || rz < 0 || rz >= g.nz)
                return fail(x, FWI_ERR_GEOMETRY, "shot " + std::to_string(s) + ": receiver " + std::to_string(r) + " outside the model");
            recs[s][r] = {(long long)(rz + g.z0p) * g.ld + rx + g.x0p, syn_off + (long long)r * d.nt0};
        }
        tr_syn_off[s] = syn_off;
        tr0[s] = (int)geo.size();
        tr_nr[s] = sh.nr;
        tr_nt0[s] = d.nt0;
        for (int r = 0; r < sh.nr; ++r)
            geo.push_back(make_float4(sh.src_x, sh.src_z, sh.rec_xz[2 * r], sh.rec_xz[2 * r + 1]));
        syn_off += (long long)sh.nr * d.nt0;
    }
    // slots: shots sorted by nt, longest first, so the active shots of a step form a prefix
    std::vector<int> order(nshots);
    for (int s = 0; s < nshots; ++s) order[s] = s;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return sd[a].nt > sd[b].nt; });

    free_shots(x);
    const long long strip_len = 2LL * x->S * (g.nx + g.nz);
    {
        const int nt_run = sd[order[0]].nt;
        const long long half_b = (long long)nshots * g.fstride * 4, phalf_b = (long long)nshots * x->pl.stride * 4;
        long long strips_b = 0;
        for (int s = 0; s < nshots; ++s) strips_b += (long long)sd[s].nt * strip_len * 4;
        const long long base_b = 5 * half_b + 4 * phalf_b + 4 * (3 * syn_off + wav_tot);
        const int r = choose_store(x, nshots, nt_run, base_b, strips_b);
        if (r) return r;
    }
    std::vector<ShotDev> slot(nshots);
    std::vector<RecSample> samp;
    std::vector<RecDev> rec_all;
    std::vector<int> rt_all;
    std::vector<float> wav_all(wav_tot);
    std::vector<RecCell8> cells8;
    std::vector<long long> rec8;
    x->cell8_off.assign(nshots + 1, 0);
    long long ring_off = 0;
    const int ntiles = g.ntx * g.ntz;
    x->nt_slot.resize(nshots);
    x->samp_off.assign(nshots + 1, 0);
    for (int k = 0; k < nshots; ++k) {
        const int s = order[k];
        ShotDev d = sd[s];
        d.ring_off = ring_off;
        ring_off += (long long)(x->store == FWI_STORE_STRIPS ? d.nt : x->seg + 2) * strip_len;
        // sampling: one entry per receiver; injection: receivers grouped by
        // tile (CSR), summed inside the tile in receiver order
        std::vector<std::pair<int, RecDev>> tmp;
        for (size_t r = 0; r < recs[s].size(); ++r) {
            const long long foff = recs[s][r].foff;
            samp.push_back(RecSample{k, 0, foff, recs[s][r].syn_base, 0});
            const int row = (int)(foff / g.ld), col = (int)(foff % g.ld);
            const int cx = col - g.xoff, rz = row - g.zoff;  // relative to the tile grid's origin (>= 0)
            RecDev rd{};
            rd.cell = (rz % TZ) * TX + (cx % TX);
            rd.syn_base = recs[s][r].syn_base;
            tmp.push_back({(rz / TZ) * g.ntx + cx / TX, rd});
        }
        // by tile, then by cell; stable, so receivers that share a cell keep their
        // input order and the backward sums them in that fixed order
        std::stable_sort(tmp.begin(), tmp.end(), [](const auto& a, const auto& b2) {
            return a.first != b2.first ? a.first < b2.first : a.second.cell < b2.second.cell;
        });
        d.rtile_off = (int)rt_all.size();
        {
            std::vector<int> cnt(ntiles + 1, 0);
            for (auto& t : tmp) cnt[t.first + 1]++;
            for (int t = 0; t < ntiles; ++t) cnt[t + 1] += cnt[t];
            const int rbase = (int)rec_all.size();
            for (int t = 0; t <= ntiles; ++t) rt_all.push_back(cnt[t] + rbase);
            for (auto& t : tmp) rec_all.push_back(t.second);
        }
        x->samp_off[k + 1] = (int)samp.size();
        if (x->M == 4) {           // receiver cells of the 8th-order injection: by cell, input order inside
            std::vector<int> ord(recs[s].size());
            for (size_t r = 0; r < ord.size(); ++r) ord[r] = (int)r;
            std::stable_sort(ord.begin(), ord.end(), [&](int a, int b2) { return recs[s][a].foff < recs[s][b2].foff; });
            for (size_t q = 0; q < ord.size(); ++q) {
                const Rec& rr = recs[s][ord[q]];
                if (q == 0 || rr.foff != recs[s][ord[q - 1]].foff)
                    cells8.push_back(RecCell8{k, (int)rec8.size(), 0, 0, rr.foff});
                ++cells8.back().count;
                rec8.push_back(rr.syn_base);
            }
            x->cell8_off[k + 1] = (int)cells8.size();
        }
        std::memcpy(&wav_all[wav_off[s]], shots[s].wavelet, sizeof(float) * shots[s].nt);
        slot[k] = d;
        x->nt_slot[k] = d.nt;
    }
    x->nshots = nshots;
    x->nt_run = x->nt_slot[0];
    x->nsamples = syn_off;
    x->npartial = (int)std::min<long long>(1024, std::max<long long>(1, (syn_off + 255) / 256));
    size_t& b = x->bytes_shots;
    const size_t half = (size_t)nshots * g.fstride, phalf = (size_t)nshots * x->pl.stride;
    int e = 0;
    e = e ? e : dalloc(x, &x->F, 2 * half, &b);
    e = e ? e : dalloc(x, &x->A, 2 * half, &b);
    e = e ? e : dalloc(x, &x->Gacc, half, &b);
    e = e ? e : dalloc(x, &x->psiF, 2 * phalf, &b);
    e = e ? e : dalloc(x, &x->psiA, 2 * phalf, &b);
    e = e ? e : dalloc(x, &x->ring, (size_t)ring_off, &b);
    e = e ? e : dalloc(x, &x->syn, (size_t)syn_off, &b);
    e = e ? e : dalloc(x, &x->res, (size_t)syn_off, &b);
    e = e ? e : dalloc(x, &x->obs, (size_t)syn_off, &b);
    e = e ? e : dalloc(x, &x->wav, (size_t)wav_tot, &b);
    e = e ? e : dalloc(x, &x->shots_d, (size_t)nshots, &b);
    e = e ? e : dalloc(x, &x->samp_d, samp.size(), &b);
    e = e ? e : dalloc(x, &x->recs_d, rec_all.size(), &b);
    e = e ? e : dalloc(x, &x->rtile_d, rt_all.size(), &b);
    e = e ? e : dalloc(x, &x->partial, (size_t)x->npartial, &b);
    e = e ? e : dalloc(x, &x->mis, 2, &b);
    e = e ? e : dalloc(x, &x->geo_d, geo.size(), &b);
    e = e ? e : dalloc(x, &x->xpart_d, geo.size(), &b);
    if (!e && x->M == 4) {
        e = dalloc(x, &x->X8, 4 * half, &b);
        e = e ? e : dalloc(x, &x->cells8_d, cells8.size(), &b);
        e = e ? e : dalloc(x, &x->rec8_d, rec8.size(), &b);
        x->ncell8 = (int)cells8.size();
    }
    if (!e && x->nsnap > 0) {
        const size_t nblk = (size_t)x->nsnap * nshots;
        const size_t elem = x->cfg.snap_precision == FWI_SNAP_F32 ? 4 : 2;
        unsigned char* sp = nullptr;
        e = dalloc(x, &sp, nblk * 2 * g.fstride * elem, &b);
        x->snapP = sp;
        e = e ? e : dalloc(x, &x->snapPsi, nblk * x->pl.stride, &b);
        e = e ? e : dalloc(x, &x->snapAmax, nblk * 2, &b);
    }
    if (e) { std::string m = x->err; free_shots(x); x->err = m; return e; }
    x->stats.store = x->store;
    x->stats.segments = x->nseg;
    x->stats.device_bytes = (long long)(x->bytes_model + x->bytes_shots);
    x->store_bytes = (long long)ring_off * 4 +
                     (x->nsnap > 0 ? (long long)x->nsnap * nshots *
                                         (2 * g.fstride * (x->cfg.snap_precision == FWI_SNAP_F32 ? 4 : 2) +
                                          4 * x->pl.stride + 8) : 0);
    x->stats.store_bytes = x->store_bytes;
    for (int h = 0; h < 2; ++h)
        if (encode_field_map(&x->tm_F[h], x->F + h * half, g, x->rows_alloc, nshots) ||
            encode_field_map(&x->tm_A[h], x->A + h * half, g, x->rows_alloc, nshots)) {
            free_shots(x);
            return fail(x, FWI_ERR_CUDA, "cuTensorMapEncodeTiled failed for a field");
        }
    CK(cudaMemcpyAsync(x->shots_d, slot.data(), sizeof(ShotDev) * nshots, cudaMemcpyHostToDevice, x->st));
    if (!samp.empty()) {
        CK(cudaMemcpyAsync(x->samp_d, samp.data(), sizeof(RecSample) * samp.size(), cudaMemcpyHostToDevice, x->st));
        CK(cudaMemcpyAsync(x->recs_d, rec_all.data(), sizeof(RecDev) * rec_all.size(), cudaMemcpyHostToDevice, x->st));
    }
    CK(cudaMemcpyAsync(x->rtile_d, rt_all.data(), sizeof(int) * rt_all.size(), cudaMemcpyHostToDevice, x->st));
    if (x->M == 4) {
        // zero buffers: positions a pass never writes (outside its range) read as 0
        CK(cudaMemsetAsync(x->X8, 0, sizeof(float) * 4 * half, x->st));
        if (!cells8.empty()) {
            CK(cudaMemcpyAsync(x->cells8_d, cells8.data(), sizeof(RecCell8) * cells8.size(), cudaMemcpyHostToDevice, x->st));
            CK(cudaMemcpyAsync(x->rec8_d, rec8.data(), sizeof(long long) * rec8.size(), cudaMemcpyHostToDevice, x->st));
        }
    }
    CK(cudaMemcpyAsync(x->wav, wav_all.data(), sizeof(float) * wav_all.size(), cudaMemcpyHostToDevice, x->st));
    if (!geo.empty()) CK(cudaMemcpyAsync(x->geo_d, geo.data(), sizeof(float4) * geo.size(), cudaMemcpyHostToDevice, x->st));
    x->shot_syn_off = tr_syn_off;
    x->shot_tr0 = tr0;
    x->shot_nr = tr_nr;
    x->shot_nt0 = tr_nt0;
    x->ntraces = (int)geo.size();
    if (x->msf.kind == FWI_MISFIT_XCORR && xcorr_too_long(x)) {
        free_shots(x);
        return fail(x, FWI_ERR_ARG, "traces too long for the XCORR kernel");
    }
    CK(cudaMemsetAsync(x->syn, 0, sizeof(float) * std::max<long long>(1, syn_off), x->st));
#ifdef FWI_SELF_CHECK
    {
        DbgRanges r{};
        auto add = [&](const void* p, size_t bytes) {
            if (p && r.n < 24) { r.lo[r.n] = (unsigned long long)p; r.hi[r.n] = (unsigned long long)p + bytes; ++r.n; }
        };
        add(x->F, sizeof(float) * 2 * half); add(x->A, sizeof(float) * 2 * half); add(x->Gacc, sizeof(float) * half);
        add(x->psiF, sizeof(float) * 2 * phalf); add(x->psiA, sizeof(float) * 2 * phalf);
        add(x->ring, sizeof(float) * ring_off); add(x->syn, sizeof(float) * syn_off); add(x->res, sizeof(float) * syn_off);
        add(x->obs, sizeof(float) * syn_off); add(x->wav, sizeof(float) * wav_tot);
        add(x->shots_d, sizeof(ShotDev) * nshots); add(x->samp_d, sizeof(RecSample) * samp.size());
        add(x->recs_d, sizeof(RecDev) * rec_all.size()); add(x->rtile_d, sizeof(int) * rt_all.size());
        add(x->K, sizeof(float) * g.fstride); add(x->vel, sizeof(float) * g.nx * g.nz); add(x->gen_d, sizeof(int2) * x->ngen);
        add(x->pmlc, sizeof(float) * 8 * (2 * g.npml + 1));
        CK(cudaMemcpyToSymbol(g_dbg, &r, sizeof(r)));
        fprintf(stderr, "FWI diag: %d ranges\n", r.n);
    }
#endif
    return finish(x);
}

int fwi_set_observed(fwi_ctx* x, const float* obs)
{
    if (!x || !obs) return fail(x, FWI_ERR_ARG, "null argument");
    if (!x->nshots) return fail(x, FWI_ERR_STATE, "fwi_set_shots first");
    CK(cudaSetDevice(x->cfg.device));
    CK(cudaMemcpyAsync(x->obs, obs, sizeof(float) * x->nsamples, cudaMemcpyHostToDevice, x->st));
    int s = finish(x);
    if (s) return s;
    x->have_obs = true;
    return FWI_OK;
}

static void record_stats(fwi_ctx* x, bool fwd, bool mis, bool bwd)
{
    long long cells = 0;
    for (int nt : x->nt_slot) cells += (long long)nt;
    const double cs = (double)cells * x->g.nx * x->g.nz;
    x->stats.ms_forward = fwd ? event_ms(x->ev[0], x->ev[1]) : 0.0;
    x->stats.ms_misfit = mis ? event_ms(x->ev[4], x->ev[5]) : 0.0;
    x->stats.ms_backward = bwd ? event_ms(x->ev[2], x->ev[3]) : 0.0;
    x->stats.ms_total = event_ms(x->ev[6], x->ev[7]);
    x->stats.cell_steps = cs * ((fwd ? 1 : 0) + (bwd ? 2 : 0));
    x->stats.device_bytes = (long long)(x->bytes_model + x->bytes_shots);
    x->stats.store = x->store;
    x->stats.segments = x->nseg;
    x->stats.store_bytes = x->store_bytes;
}

int fwi_forward(fwi_ctx* x, float* syn_out)
{
    if (!x) return FWI_ERR_ARG;
    if (usable(x)) return FWI_ERR_STATE;
    if (!x->have_model || !x->nshots) return fail(x, FWI_ERR_STATE, "fwi_set_model and fwi_set_shots first");
    CK(cudaSetDevice(x->cfg.device));
    CK(cudaEventRecord(x->ev[6], x->st));
    int s = run_phase(x, PH_FWD, false);
    if (s) return s;
    if (syn_out) CK(cudaMemcpyAsync(syn_out, x->syn, sizeof(float) * x->nsamples, cudaMemcpyDeviceToHost, x->st));
    CK(cudaEventRecord(x->ev[7], x->st));
    s = finish(x);
    if (s) return s;
    record_stats(x, true, false, false);
    x->have_fwd = true;
    return FWI_OK;
}

int fwi_backward(fwi_ctx* x, const float* residual, double* grad_out)
{
    if (!x || !residual) return fail(x, FWI_ERR_ARG, "null argument");
    if (usable(x)) return FWI_ERR_STATE;
    if (!x->have_fwd) return fail(x, FWI_ERR_STATE, "fwi_forward on the current model first");
    CK(cudaSetDevice(x->cfg.device));
    CK(cudaEventRecord(x->ev[6], x->st));
    CK(cudaMemcpyAsync(x->res, residual, sizeof(float) * x->nsamples, cudaMemcpyHostToDevice, x->st));
    x->stats.launches = 0;
    int s = run_phase(x, PH_BWD, false);
    if (s) return s;
    if (grad_out)
        CK(cudaMemcpyAsync(grad_out, x->grad, sizeof(double) * x->g.nx * x->g.nz, cudaMemcpyDeviceToHost, x->st));
    CK(cudaEventRecord(x->ev[7], x->st));
    s = finish(x);
    x->have_fwd = false;   // the rebuild consumed the final forward fields
    if (s) return s;
    record_stats(x, false, false, true);
    return FWI_OK;
}

// obs_ready: an event the misfit phase waits for (fwi_gradient_obs's upload), or null
static int gradient_impl(fwi_ctx* x, double* misfit, cudaEvent_t obs_ready = nullptr)
{
    if (!x) return FWI_ERR_ARG;
    if (usable(x)) return FWI_ERR_STATE;
    if (!x->have_model || !x->nshots || !x->have_obs)
        return fail(x, FWI_ERR_STATE, "fwi_set_model, fwi_set_shots and fwi_set_observed first");
    CK(cudaSetDevice(x->cfg.device));
    x->have_fwd = false;
    CK(cudaEventRecord(x->ev[6], x->st));
#ifdef FWI_SELF_CHECK
    const bool graph = false;          // DIAG_SYNC synchronises after every launch
#else
    const bool graph = x->cfg.use_graph != 0;
#endif
    int s = run_phase(x, PH_FWD, graph);
    if (!s && obs_ready) CK(cudaStreamWaitEvent(x->st, obs_ready, 0));
    if (!s) s = run_phase(x, PH_MIS, graph);
    if (!s) s = run_phase(x, PH_BWD, graph);
    if (s) return s;
    if (graph) x->stats.launches = x->graph_launches[0] + x->graph_launches[1] + x->graph_launches[2];
    if (misfit) CK(cudaMemcpyAsync(misfit, x->mis, 2 * sizeof(double), cudaMemcpyDeviceToHost, x->st));
    return FWI_OK;
}

int fwi_gradient(fwi_ctx* x, double* misfit, double* grad_out)
{
    int s = gradient_impl(x, misfit);
    if (s) return s;
    if (grad_out)
        CK(cudaMemcpyAsync(grad_out, x->grad, sizeof(double) * x->g.nx * x->g.nz, cudaMemcpyDeviceToHost, x->st));
    CK(cudaEventRecord(x->ev[7], x->st));
    s = finish(x);
    if (s) return s;
    record_stats(x, true, true, true);
    return FWI_OK;
}

static int gradient_obs_impl(fwi_ctx* x, const float* obs, double* misfit, double* grad_out)
{
    if (!x->have_model || !x->nshots) return fail(x, FWI_ERR_STATE, "fwi_set_model and fwi_set_shots first");
    CK(cudaSetDevice(x->cfg.device));
    // the upload starts after the work already queued on the stream (the last misfit
    // phase read obs) and runs beside the forward phase, which does not read it
    CK(cudaEventRecord(x->obs_ev, x->st));
    CK(cudaStreamWaitEvent(x->obs_st, x->obs_ev, 0));
    CK(cudaMemcpyAsync(x->obs, obs, sizeof(float) * x->nsamples, cudaMemcpyHostToDevice, x->obs_st));
    CK(cudaEventRecord(x->obs_ev, x->obs_st));
    x->have_obs = true;
    int s = gradient_impl(x, misfit, x->obs_ev);
    if (s) return s;
    if (grad_out)
        CK(cudaMemcpyAsync(grad_out, x->grad, sizeof(double) * x->g.nx * x->g.nz, cudaMemcpyDeviceToHost, x->st));
    CK(cudaEventRecord(x->ev[7], x->st));
    s = finish(x);
    if (s) return s;
    record_stats(x, true, true, true);
    return FWI_OK;
}

int fwi_gradient_obs(fwi_ctx* x, const float* obs, double* misfit, double* grad_out)
{
    if (!x || !obs) return fail(x, FWI_ERR_ARG, "null argument");
    if (usable(x)) return FWI_ERR_STATE;
    int s = gradient_obs_impl(x, obs, misfit, grad_out);
    // the host buffer is the caller's again on return, on every path
    cudaError_t e = cudaStreamSynchronize(x->obs_st);
    if (!s && e != cudaSuccess) s = cuda_fail(x, e, "fwi_gradient_obs upload");
    return s;
}

int fwi_gradient_f32(fwi_ctx* x, double* misfit, float* grad_out)
{
    int s = gradient_impl(x, misfit);
    if (s) return s;
    const long long n = (long long)x->g.nx * x->g.nz;
    if (grad_out) {
        FWI_LAUNCH(k_to_float, 256, 256, 0, x->st, x->grad, x->gradf, n);
        CK(cudaGetLastError());
        CK(cudaMemcpyAsync(grad_out, x->gradf, sizeof(float) * n, cudaMemcpyDeviceToHost, x->st));
    }
    CK(cudaEventRecord(x->ev[7], x->st));
    s = finish(x);
    if (s) return s;
    record_stats(x, true, true, true);
    return FWI_OK;
}

const double* fwi_grad_device(const fwi_ctx* x) { return x ? x->grad : nullptr; }

// Device address of g_noalloc_trace_sums on the current device.  The first
// call on a device looks it up (cudaGetSymbolAddress, with that device
// current) and keeps it.  Later calls look it up again whenever `st` is not
// being captured, because a cudaDeviceReset reloads the module and may move
// the array; during a capture they use the kept address, so the first call on
// a device has to come before any capture.
static double* noalloc_scratch(int device, cudaStream_t st, cudaError_t* err)
{
    static std::mutex m;
    static double* addr[64] = {};
    *err = cudaSuccess;
    if (device < 0 || device >= 64) { *err = cudaErrorInvalidDevice; return nullptr; }
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    *err = cudaStreamIsCapturing(st, &cap);
    if (*err != cudaSuccess) return nullptr;
    std::lock_guard<std::mutex> lk(m);
    if (!addr[device] || cap == cudaStreamCaptureStatusNone) {
        double* p = nullptr;
        *err = cudaGetSymbolAddress((void**)&p, g_noalloc_trace_sums);
        if (*err != cudaSuccess) return nullptr;
        addr[device] = p;
    }
    return addr[device];
}

int fwi_l2_misfit_noalloc(const float* syn, const float* obs, float* residual, int ntraces, int nsamples,
                          double* misfit, void* stream)
{
    if (!syn || !obs || !residual || !misfit || ntraces < 1 || nsamples < 1) return FWI_ERR_ARG;
    if (ntraces > FWI_NOALLOC_MAX_TRACES) return FWI_ERR_ARG;   // beyond the static scratch
    // An error already pending on this thread belongs to the caller: leave it
    // for them to read and launch nothing.
    if (cudaPeekAtLastError() != cudaSuccess) return FWI_ERR_CUDA;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) { cudaGetLastError(); return FWI_ERR_NODEVICE; }
    cudaStream_t st = (cudaStream_t)stream;
    cudaError_t e = cudaSuccess;
    double* part = noalloc_scratch(dev, st, &e);
    if (!part) { cudaGetLastError(); return FWI_ERR_CUDA; }
    FWI_LAUNCH(k_misfit_traces, ntraces, 256, 0, st, syn, obs, residual, nsamples, part);
    if (cudaGetLastError() != cudaSuccess) return FWI_ERR_CUDA;     // this call's own launch error
    FWI_LAUNCH(k_misfit_final, 1, 256, 0, st, part, ntraces, misfit);
    if (cudaGetLastError() != cudaSuccess) return FWI_ERR_CUDA;
    return FWI_OK;
}

int fwi_set_misfit(fwi_ctx* x, const fwi_misfit* m)
{
    if (!x || !m) return FWI_ERR_ARG;
    if (m->kind != FWI_MISFIT_L2 && m->kind != FWI_MISFIT_XCORR)
        return fail(x, FWI_ERR_ARG, "unknown misfit kind");
    if (m->kind == FWI_MISFIT_XCORR && m->slice != FWI_XCORR_MIDDLE && m->slice != FWI_XCORR_LEADING)
        return fail(x, FWI_ERR_ARG, "unknown XCORR slice");
    CK(cudaSetDevice(x->cfg.device));
    if (m->kind == FWI_MISFIT_XCORR) {
        if (xcorr_too_long(x)) return fail(x, FWI_ERR_ARG, "traces too long for the XCORR kernel");
        CK(xcorr_setup());
    }
    x->msf = *m;
    // the captured misfit phase depends on the kind
    if (x->gexec[1]) { cudaGraphExecDestroy(x->gexec[1]); x->gexec[1] = nullptr; }
    if (x->graph[1]) { cudaGraphDestroy(x->graph[1]); x->graph[1] = nullptr; }
    x->have_fwd = false;
    return FWI_OK;
}

int fwi_set_stream(fwi_ctx* x, void* stream)
{
    if (!x) return FWI_ERR_ARG;
    CK(cudaSetDevice(x->cfg.device));
    CK(cudaStreamSynchronize(x->st));
    x->st = stream ? (cudaStream_t)stream : x->own;
    return FWI_OK;
}

int fwi_set_tuning(fwi_ctx* x, const fwi_tuning* t)
{
    if (!x || !t) return FWI_ERR_ARG;
    for (int i = 0; i < 5; ++i)
        if (t->reserved[i]) return fail(x, FWI_ERR_ARG, "fwi_tuning.reserved must be zero");
    const fwi_tuning d = default_tuning(x);
    fwi_tuning n = x->tune;
    auto pick = [](int v, int cur) { return v ? v : cur; };
    n.x_first = t->x_first ? t->x_first : d.x_first;
    n.z_first = t->z_first ? t->z_first : d.z_first;
    n.fwd_gen_blocks = pick(t->fwd_gen_blocks, d.fwd_gen_blocks);
    n.bwd_gen_blocks = pick(t->bwd_gen_blocks, d.bwd_gen_blocks);
    n.fwd_int_blocks = pick(t->fwd_int_blocks, d.fwd_int_blocks);
    n.bwd_int_blocks = pick(t->bwd_int_blocks, d.bwd_int_blocks);
    n.class_order = pick(t->class_order, d.class_order);
    n.serial = pick(t->serial, d.serial);
    n.priority = pick(t->priority, d.priority);
    n.gen_grid = pick(t->gen_grid, d.gen_grid);
    n.bwd_zgen_blocks = pick(t->bwd_zgen_blocks, d.bwd_zgen_blocks);
    const Geo& g = x->g;
    if (n.x_first < d.x_first || n.x_first % 4 || n.x_first >= g.pnx - g.npml - 4)
        return fail(x, FWI_ERR_ARG, "x_first must be a multiple of 4 from " + std::to_string(d.x_first));
    if (n.z_first < d.z_first || n.z_first % R || n.z_first >= g.pnz - 4)
        return fail(x, FWI_ERR_ARG, "z_first must be a multiple of 4 from " + std::to_string(d.z_first));
    if ((n.fwd_gen_blocks != 3 && n.fwd_gen_blocks != 4) || (n.bwd_gen_blocks != 3 && n.bwd_gen_blocks != 4) ||
        (n.fwd_int_blocks != 4 && n.fwd_int_blocks != 6) || (n.bwd_int_blocks != 3 && n.bwd_int_blocks != 4) ||
        (n.class_order != 1 && n.class_order != 2) || (n.serial != 1 && n.serial != 2) ||
        (n.priority != 1 && n.priority != 2) || n.gen_grid < 1 || n.gen_grid > 5 ||
        (n.bwd_zgen_blocks != 3 && n.bwd_zgen_blocks != 4))
        return fail(x, FWI_ERR_ARG, "a fwi_tuning value outside its list");
    CK(cudaSetDevice(x->cfg.device));
    CK(cudaStreamSynchronize(x->st));
    const bool relayout = n.x_first != x->tune.x_first || n.z_first != x->tune.z_first;
    const bool reprio = n.priority != x->tune.priority;
    x->tune = n;
    drop_graph(x);                       // the captured phases hold the old launches
    if (reprio) CK(make_side_streams(x));
    if (relayout) {
        free_shots(x);
        x->have_model = false;
        if (int st = set_layout(x)) return st;
    }
    return FWI_OK;
}

int fwi_get_tuning(const fwi_ctx* x, fwi_tuning* out)
{
    if (!x || !out) return FWI_ERR_ARG;
    *out = x->tune;
    return FWI_OK;
}

int fwi_time_steps(fwi_ctx* x, int steps, double* ms_fwd, double* ms_bwd)
{
    if (!x || steps < 1 || !ms_fwd || !ms_bwd) return FWI_ERR_ARG;
    if (usable(x)) return FWI_ERR_STATE;
    if (!x->have_model || !x->nshots) return fail(x, FWI_ERR_STATE, "fwi_set_model and fwi_set_shots first");
    CK(cudaSetDevice(x->cfg.device));
    const long long half = (long long)x->nshots * x->g.fstride;
    const long long phalf = (long long)x->nshots * x->pl.stride;
    // backward steps from the end of the record read the strips the ring holds
    // for them: with checkpoints, those of the last segment
    const int last_seg = x->nt_run - (x->nseg - 1) * x->seg;
    const int nf = std::min(steps, x->nt_run);
    const int nb = std::min(steps, x->store == FWI_STORE_SNAPSHOTS ? last_seg : x->nt_run);
    x->have_fwd = false;
    CK(cudaMemsetAsync(x->F, 0, sizeof(float) * 2 * half, x->st));
    CK(cudaMemsetAsync(x->psiF, 0, sizeof(float) * 2 * phalf, x->st));
    CK(cudaMemsetAsync(x->A, 0, sizeof(float) * 2 * half, x->st));
    CK(cudaMemsetAsync(x->psiA, 0, sizeof(float) * 2 * phalf, x->st));
    StepParams P = base_params(x);
    P.gacc = x->Gacc + x->origin;
    set_ring(x, P, x->nseg - 1);
    // The steps are captured into two CUDA graphs and the replay is timed, as
    // the gradient replays its phases (direct launches time differently);
    // without capture (diagnostics builds, the CPU emulation) they run directly.
    cudaGraph_t gr[2] = {nullptr, nullptr};
    cudaGraphExec_t ge[2] = {nullptr, nullptr};
    bool graphs = false;
#ifndef FWI_SELF_CHECK
    graphs = true;
    for (int ph = 0; ph < 2 && graphs; ++ph) {
        if (cudaStreamBeginCapture(x->st, cudaStreamCaptureModeThreadLocal) != cudaSuccess) { graphs = false; break; }
        if (ph == 0) forward_steps(x, P, 0, nf, 0, x->nshots, false);
        else backward_steps(x, P, x->nt_run, x->nt_run - nb, 0, x->nshots);
        if (cudaStreamEndCapture(x->st, &gr[ph]) != cudaSuccess ||
            cudaGraphInstantiate(&ge[ph], gr[ph], 0) != cudaSuccess)
            graphs = false;
    }
    cudaGetLastError();                       // a failed capture falls back to direct launches
#endif
    auto run = [&](int ph) {
        if (graphs) return cudaGraphLaunch(ge[ph], x->st);
        if (ph == 0) forward_steps(x, P, 0, nf, 0, x->nshots, false);
        else backward_steps(x, P, x->nt_run, x->nt_run - nb, 0, x->nshots);
        return cudaGetLastError();
    };
    cudaError_t e = run(0);                   // warm replay: module loads, caches
    if (e == cudaSuccess) e = run(1);
    if (e == cudaSuccess) e = cudaEventRecord(x->ev[0], x->st);
    if (e == cudaSuccess) e = run(0);
    if (e == cudaSuccess) e = cudaEventRecord(x->ev[1], x->st);
    if (e == cudaSuccess) e = run(1);
    if (e == cudaSuccess) e = cudaEventRecord(x->ev[2], x->st);
    for (int ph = 0; ph < 2; ++ph) {
        if (ge[ph]) cudaGraphExecDestroy(ge[ph]);
        if (gr[ph]) cudaGraphDestroy(gr[ph]);
    }
    if (e != cudaSuccess) return cuda_fail(x, e, "fwi_time_steps");
    int s = finish(x);
    if (s) return s;
    *ms_fwd = event_ms(x->ev[0], x->ev[1]) / nf;
    *ms_bwd = event_ms(x->ev[1], x->ev[2]) / nb;
    return FWI_OK;
}

int fwi_get_stats(const fwi_ctx* x, fwi_stats* out)
{
    if (!x || !out) return FWI_ERR_ARG;
    *out = x->stats;
    return FWI_OK;
}

}  // extern "C"
