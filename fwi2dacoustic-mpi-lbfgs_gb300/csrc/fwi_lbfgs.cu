// fwi_lbfgs.cu -- the L-BFGS driver of MBotOpt.c (MBotOpt.c:55-214) as a
// device optimizer with reverse communication: the caller evaluates the
// objective and its gradient at the point the optimizer hands out, the
// optimizer takes one line-search decision per evaluation.  All vectors
// (x, the saved xp / gp, the direction d and the m correction pairs s, y)
// live in HBM in FP64; dot products are deterministic two-pass FP64
// reductions.  The host waits only for the values the line search decides
// on (the slopes g.d, |x| and |g|) and for the trial point it hands out; the
// two-loop recursion keeps its coefficients on the device.  The decisions, step rules and two-loop recursion are those
// of MBotOpt.c (see fwi_gb300.h).
#include "fwi_gb300.h"
#ifdef FWI_CPU_EMU
#include "cpu_emu.h"
#else
#include <cuda_runtime.h>
#include "cpu_emu.h"
#endif

#include <cmath>
#include <vector>

namespace {

#ifdef FWI_CPU_EMU
constexpr int DOT_BLOCKS = 2;         // the CPU emulation runs blocks one after another
#else
constexpr int DOT_BLOCKS = 608;       // 4 x 152 SMs
#endif
constexpr int DOT_THREADS = 256;

__global__ void k_dot_part(const double* __restrict__ a, const double* __restrict__ b, long long n,
                           double* __restrict__ part)
{
    __shared__ double red[DOT_THREADS / 32];
    double s = 0;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        s += a[i] * b[i];
    for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0;
        for (int w = 0; w < DOT_THREADS / 32; ++w) t += red[w];
        part[blockIdx.x] = t;
    }
}

__global__ void k_dot_final(const double* __restrict__ part, int n, double* __restrict__ out)
{
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        double t = 0;
        for (int i = 0; i < n; ++i) t += part[i];
        *out = t;
    }
}

// y = -x (the previous contents of y are not read: they may be uninitialised)
__global__ void k_neg(double* __restrict__ y, const double* __restrict__ x, long long n)
{
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        y[i] = -x[i];
}

// The two-loop recursion with its coefficients in device memory, so that its
// dot products need no host round trip: sc = {dot, ys[m], yy, alpha[m]}.
// First loop:  alpha_j = dot / ys_j (kept for the second loop); d = -alpha_j y_j + d.
__global__ void k_loop1(double* __restrict__ d, const double* __restrict__ yj, double* __restrict__ sc, int j, int m,
                        long long n)
{
    const double a = sc[0] / sc[1 + j];
    if (blockIdx.x == 0 && threadIdx.x == 0) sc[2 + m + j] = a;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        d[i] = -a * yj[i] + 1.0 * d[i];
}
// d *= ys / yy of the newest pair (slot j)
__global__ void k_scale_pair(double* __restrict__ d, const double* __restrict__ sc, int j, int m, long long n)
{
    const double c = sc[1 + j] / sc[1 + m];
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        d[i] *= c;
}
// Second loop: beta = dot / ys_j; d = (alpha_j - beta) s_j + d.
__global__ void k_loop2(double* __restrict__ d, const double* __restrict__ sj, const double* __restrict__ sc, int j,
                        int m, long long n)
{
    const double c = sc[2 + m + j] - sc[0] / sc[1 + j];
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        d[i] = c * sj[i] + 1.0 * d[i];
}

// z = x + c * y
__global__ void k_xpcy(double* __restrict__ z, const double* __restrict__ x, const double* __restrict__ y, double c,
                       long long n)
{
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        z[i] = x[i] + c * y[i];
}

}  // namespace

struct fwi_lbfgs {
    long long n = 0;
    fwi_lbfgs_param p{};
    double *x = nullptr, *xp = nullptr, *g = nullptr, *gp = nullptr, *d = nullptr, *S = nullptr, *Y = nullptr;
    double *part = nullptr, *dot = nullptr;
    double* sc = nullptr;          // device scalars of the two-loop recursion: dot, ys[m], yy, alpha[m]
    std::vector<double> step_arr;
    int k = 1, end = 0, count = 0, evaluations = 0, state = -1;
    double step = 0, fx = 0, finit = 0, dginit = 0, dgtest = 0;
    cudaStream_t st = nullptr;
};

namespace {

const fwi_lbfgs_param kDefaults = {12, 1e-9, 8, 6, 1e-7, 0.98};   // lbfgs.h:77-79

#ifdef FWI_CPU_EMU
unsigned vec_blocks(long long n) { return (unsigned)std::min<long long>((n + 255) / 256, 2); }
#else
unsigned vec_blocks(long long n) { return (unsigned)std::min<long long>((n + 255) / 256, 4 * 152 * 8); }
#endif

// a . b into the device scalar *dev (no host wait)
void dot_dev(fwi_lbfgs* L, const double* a, const double* b, double* dev)
{
    FWI_LAUNCH(k_dot_part, DOT_BLOCKS, DOT_THREADS, 0, L->st, a, b, L->n, L->part);
    FWI_LAUNCH(k_dot_final, 1, 32, 0, L->st, L->part, DOT_BLOCKS, dev);
}

// a . b on the host (one wait): for the line-search decisions
int dot(fwi_lbfgs* L, const double* a, const double* b, double* out)
{
    FWI_LAUNCH(k_dot_part, DOT_BLOCKS, DOT_THREADS, 0, L->st, a, b, L->n, L->part);
    FWI_LAUNCH(k_dot_final, 1, 32, 0, L->st, L->part, DOT_BLOCKS, L->dot);
    if (cudaMemcpyAsync(out, L->dot, sizeof(double), cudaMemcpyDeviceToHost, L->st) != cudaSuccess ||
        cudaStreamSynchronize(L->st) != cudaSuccess) {
        cudaGetLastError();
        return FWI_ERR_CUDA;
    }
    return FWI_OK;
}

#define LB_CK(call) do { int s_ = (call); if (s_) return s_; } while (0)
#define LB_CU(call) do { if ((call) != cudaSuccess) { cudaGetLastError(); return FWI_ERR_CUDA; } } while (0)

int load_gradient(fwi_lbfgs* L, const double* g, int on_device)
{
    LB_CU(cudaMemcpyAsync(L->g, g, sizeof(double) * L->n, on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                          L->st));
    return FWI_OK;
}

// x = xp + step * d, handed to the caller
int trial_point(fwi_lbfgs* L, double* x_host)
{
    FWI_LAUNCH(k_xpcy, vec_blocks(L->n), 256, 0, L->st, L->x, L->xp, L->d, L->step, L->n);
    LB_CU(cudaMemcpyAsync(x_host, L->x, sizeof(double) * L->n, cudaMemcpyDeviceToHost, L->st));
    LB_CU(cudaStreamSynchronize(L->st));
    return FWI_OK;
}

// Saves the position, the initial slope and value, hands out the first trial
// point of a line search (MBotOpt.c:77-96).
int start_line_search(fwi_lbfgs* L, double* x_host)
{
    LB_CU(cudaMemcpyAsync(L->xp, L->x, sizeof(double) * L->n, cudaMemcpyDeviceToDevice, L->st));
    LB_CU(cudaMemcpyAsync(L->gp, L->g, sizeof(double) * L->n, cudaMemcpyDeviceToDevice, L->st));
    L->count = 0;
    LB_CK(dot(L, L->g, L->d, &L->dginit));
    L->finit = L->fx;
    L->dgtest = L->p.ftol * L->dginit;
    L->state = FWI_LBFGS_EVALUATE;
    return trial_point(L, x_host);
}

}  // namespace

extern "C" {

fwi_lbfgs* fwi_lbfgs_create(long long n, const fwi_lbfgs_param* param, int* status)
{
    auto bail = [&](int s, fwi_lbfgs* L) -> fwi_lbfgs* {
        if (status) *status = s;
        fwi_lbfgs_destroy(L);
        return nullptr;
    };
    const fwi_lbfgs_param p = param ? *param : kDefaults;
    if (n < 1 || p.m < 1 || p.max_linesearch < 1 || p.max_iterations < 0) return bail(FWI_ERR_ARG, nullptr);
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) { cudaGetLastError(); return bail(FWI_ERR_NODEVICE, nullptr); }
    fwi_lbfgs* L = new fwi_lbfgs;
    L->n = n;
    L->p = p;
    double** bufs[] = {&L->x, &L->xp, &L->g, &L->gp, &L->d};
    for (double** b : bufs)
        if (cudaMalloc(b, sizeof(double) * n) != cudaSuccess) { cudaGetLastError(); return bail(FWI_ERR_NOMEM, L); }
    if (cudaMalloc(&L->S, sizeof(double) * n * p.m) != cudaSuccess ||
        cudaMalloc(&L->Y, sizeof(double) * n * p.m) != cudaSuccess ||
        cudaMalloc(&L->part, sizeof(double) * DOT_BLOCKS) != cudaSuccess || cudaMalloc(&L->dot, sizeof(double)) != cudaSuccess ||
        cudaMalloc(&L->sc, sizeof(double) * (2 + 2 * (size_t)p.m)) != cudaSuccess) {
        cudaGetLastError();
        return bail(FWI_ERR_NOMEM, L);
    }
    if (cudaStreamCreateWithFlags(&L->st, cudaStreamNonBlocking) != cudaSuccess) { cudaGetLastError(); return bail(FWI_ERR_CUDA, L); }
    L->step_arr.assign(p.max_iterations + 2, 0.0);
    if (status) *status = FWI_OK;
    return L;
}

void fwi_lbfgs_destroy(fwi_lbfgs* L)
{
    if (!L) return;
    double* bufs[] = {L->x, L->xp, L->g, L->gp, L->d, L->S, L->Y, L->part, L->dot, L->sc};
    for (double* b : bufs) if (b) cudaFree(b);
    if (L->st) cudaStreamDestroy(L->st);
    delete L;
}

int fwi_lbfgs_begin(fwi_lbfgs* L, double* x, double f, const double* g, int g_on_device, int* state)
{
    if (!L || !x || !g || !state) return FWI_ERR_ARG;
    if (!std::isfinite(f)) return FWI_ERR_NONFINITE;
    LB_CU(cudaMemcpyAsync(L->x, x, sizeof(double) * L->n, cudaMemcpyHostToDevice, L->st));
    LB_CK(load_gradient(L, g, g_on_device));
    L->fx = f;
    L->evaluations = 1;
    // d = -g, step 0.8, k = 1 (MBotOpt.c:65-74)
    FWI_LAUNCH(k_neg, vec_blocks(L->n), 256, 0, L->st, L->d, L->g, L->n);
    L->step = 0.8;
    L->k = 1;
    L->end = 0;
    std::fill(L->step_arr.begin(), L->step_arr.end(), 0.0);
    LB_CK(start_line_search(L, x));
    *state = L->state;
    return FWI_OK;
}

int fwi_lbfgs_next(fwi_lbfgs* L, double* x, double f, const double* g, int g_on_device, int* state)
{
    if (!L || !x || !g || !state) return FWI_ERR_ARG;
    if (L->state != FWI_LBFGS_EVALUATE) return FWI_ERR_STATE;
    LB_CK(load_gradient(L, g, g_on_device));
    L->fx = f;
    ++L->evaluations;
    ++L->count;
    // line-search decision (MBotOpt.c:101-151)
    const double dec = 0.5, inc = 2.1;
    double width = 0;
    bool accepted = false;
    if (f > L->finit + L->step * L->dgtest) {              // the Armijo condition fails
        width = dec;
    } else {
        double dg;
        LB_CK(dot(L, L->g, L->d, &dg));
        if (dg < L->p.wolfe * L->dginit) width = inc;
        else if (dg > -L->p.wolfe * L->dginit) width = dec;
        else accepted = true;
    }
    if (!accepted) {
        if (L->p.max_linesearch <= L->count) {
            L->state = FWI_LBFGS_MAXLINESEARCH;
            LB_CU(cudaMemcpyAsync(x, L->x, sizeof(double) * L->n, cudaMemcpyDeviceToHost, L->st));
            LB_CU(cudaStreamSynchronize(L->st));
            *state = L->state;
            return FWI_OK;
        }
        L->step *= width;
        LB_CK(trial_point(L, x));
        *state = L->state;
        return FWI_OK;
    }
    // convergence and iteration limits (MBotOpt.c:160-187)
    double xx, gg;
    LB_CK(dot(L, L->x, L->x, &xx));
    LB_CK(dot(L, L->g, L->g, &gg));
    L->step_arr[L->k] = L->step;
    if (std::sqrt(gg) / std::sqrt(xx) <= L->p.epsilon) L->state = FWI_LBFGS_SUCCESS;
    else if (L->p.max_iterations != 0 && L->p.max_iterations < L->k + 1) L->state = FWI_LBFGS_MAXITERATION;
    if (L->state != FWI_LBFGS_EVALUATE) {
        LB_CU(cudaMemcpyAsync(x, L->x, sizeof(double) * L->n, cudaMemcpyDeviceToHost, L->st));
        LB_CU(cudaStreamSynchronize(L->st));
        *state = L->state;
        return FWI_OK;
    }
    // correction pair and two-loop recursion (MBotOpt.c:188-213); its
    // coefficients stay on the device (k_loop1, k_scale_pair, k_loop2), so
    // the recursion needs no host wait
    const int m = L->p.m;
    const int newest = L->end;
    double* s = L->S + (size_t)L->end * L->n;
    double* y = L->Y + (size_t)L->end * L->n;
    const unsigned nb = vec_blocks(L->n);
    FWI_LAUNCH(k_xpcy, nb, 256, 0, L->st, s, L->x, L->xp, -1.0, L->n);
    FWI_LAUNCH(k_xpcy, nb, 256, 0, L->st, y, L->g, L->gp, -1.0, L->n);
    dot_dev(L, y, s, L->sc + 1 + newest);                  // ys of the newest pair
    dot_dev(L, y, y, L->sc + 1 + m);                       // yy
    const int bound = (m <= L->k) ? m : L->k;
    ++L->k;
    L->end = (L->end + 1) % m;
    FWI_LAUNCH(k_neg, nb, 256, 0, L->st, L->d, L->g, L->n);
    int j = L->end;
    for (int i = 0; i < bound; ++i) {
        j = (j + m - 1) % m;
        dot_dev(L, L->S + (size_t)j * L->n, L->d, L->sc);
        FWI_LAUNCH(k_loop1, nb, 256, 0, L->st, L->d, L->Y + (size_t)j * L->n, L->sc, j, m, L->n);
    }
    FWI_LAUNCH(k_scale_pair, nb, 256, 0, L->st, L->d, L->sc, newest, m, L->n);
    for (int i = 0; i < bound; ++i) {
        dot_dev(L, L->Y + (size_t)j * L->n, L->d, L->sc);
        FWI_LAUNCH(k_loop2, nb, 256, 0, L->st, L->d, L->S + (size_t)j * L->n, L->sc, j, m, L->n);
        j = (j + 1) % m;
    }
    LB_CU(cudaGetLastError());
    L->step = (L->k < 4) ? 0.2 : 0.5 * (L->step_arr[L->k - 1] + L->step_arr[L->k - 2]);
    LB_CK(start_line_search(L, x));
    *state = L->state;
    return FWI_OK;
}

int fwi_lbfgs_info(const fwi_lbfgs* L, int* iteration, double* step, int* evaluations)
{
    if (!L) return FWI_ERR_ARG;
    if (iteration) *iteration = L->k;
    if (step) *step = L->step;
    if (evaluations) *evaluations = L->evaluations;
    return FWI_OK;
}

}  // extern "C"
