// fwi_kernels8.cuh -- the 8th-order (M = 4) time stepping of the engine.
//
// The reference is 4th order only (MM 2, fwi_sys.h:7).  Its 8th-order
// extension is defined as follows (the CPU oracle states the same
// definition):
//   * a staggered first difference uses the 8th-order stencil
//       D+ at position j:  sum_k w_k (a[j+k-1] - a[j-k]),  4 <= j <= n-4
//       D- at cell i:      sum_k w_k (b[i+k] - b[i-k+1]),  3 <= i <= n-4
//     with w = (1225/1024, -245/3072, 49/5120, -5/7168) / h, wherever its 8
//     points lie inside the grid, and the reference's formulas of
//     a_lap_opt_2d_pml (fwi_2d.c:775-862: the 4th-order pair, the 2nd-order
//     edge differences, the free-surface one-sided rows) everywhere else;
//   * the CPML psi recursions are the reference's, on these differences;
//   * the rebuild's interior operator is the 8th-order stencil alone and the
//     2M-1 = 7 outer rows and columns of the physical grid are the strips.
//
// The kernels run in passes over the whole padded grid of every active shot
// (grid.z = shot slot), with the staggered quantities in HBM buffers of the
// field layout: the 8th-order path serves small grids (the 201 x 401, 8-shot
// workload: 221 x 441 padded cells, whose whole state stays in the 129 MB L2), where a
// fused tile kernel would not pay for its halo of 7 cells.  Per step:
//   forward:  k8_uv (u, v with their psi), k8_fwd (ux, vz with psi,
//             leapfrog, source, strips), then the shared receiver sampling;
//   backward: k8_adj_uv (the transposed D- and psi of the adjoint at the u/v
//             positions, and the rebuild's interior u/v of p^{m-1}),
//             k8_adj (the transposed D+, b^m without receivers), k8_inject
//             (receiver adjoint sources, one thread per receiver cell, in a
//             fixed order), k8_rebuild (p^{m-2} and the imaging).
// The transposes are gathers over the same per-position weights as the
// forward differences (w8p / w8m), so forward and adjoint share one
// definition.
#pragma once
#include "fwi_kernels.cuh"

namespace fwi {

constexpr int NSTRIP8 = 7;   // 2M-1 strips of the 8th-order rebuild

// The coefficient of a[c] in D+ at position j (n cells), the 8th-order
// definition above; top_fs: the free-surface rows of the z direction.
__device__ __forceinline__ float w8p(int j, int c, int n, const float* w, float c0, float c1, float ih, float ih840,
                                     bool top_fs)
{
    if (j < 0 || j > n) return 0.f;
    const int d = c - j;
    if (j >= 4 && j <= n - 4) {
        if (d >= 0 && d <= 3) return w[d];
        if (d >= -4 && d <= -1) return -w[-d - 1];
        return 0.f;
    }
    if (top_fs && j <= 1) {
        if (c < 0 || c > 3) return 0.f;
        const float h0[4] = {3675.f, -1225.f, 441.f, -75.f}, h1[4] = {-1085.f, 1015.f, -63.f, 5.f};
        return (j == 0 ? h0[c] : h1[c]) * ih840;
    }
    if (j >= 2 && j <= n - 2) return d == 0 ? c0 : d == -1 ? -c0 : d == 1 ? c1 : d == -2 ? -c1 : 0.f;
    if (j == 1) return c == 1 ? ih : c == 0 ? -ih : 0.f;
    if (j == n - 1) return c == n - 1 ? ih : c == n - 2 ? -ih : 0.f;
    return 0.f;
}

// The coefficient of b[j] in D- at cell i (positions 0..n).
__device__ __forceinline__ float w8m(int i, int j, int n, const float* w, float c0, float c1, float ih, float ih24,
                                     bool top_fs)
{
    if (i < 0 || i >= n) return 0.f;
    const int d = j - i;
    if (i >= 3 && i <= n - 4) {
        if (d >= 1 && d <= 4) return w[d - 1];
        if (d >= -3 && d <= 0) return -w[-d];
        return 0.f;
    }
    if (top_fs && i == 0) {
        const float h[5] = {-22.f, 17.f, 9.f, -5.f, 1.f};
        return (j >= 0 && j <= 4) ? h[j] * ih24 : 0.f;
    }
    if (i >= 1 && i <= n - 2) return d == 1 ? c0 : d == 0 ? -c0 : d == 2 ? c1 : d == -1 ? -c1 : 0.f;
    if (i == 0) return j == 1 ? ih : j == 0 ? -ih : 0.f;
    return j == n ? ih : j == n - 1 ? -ih : 0.f;
}

// D+ at position j of n values a[k * st], in the difference form (each
// stencil term is a difference, so smooth fields keep their digits).
__device__ __forceinline__ float d8p(const float* a, long long st, int n, int j, const float* w, float c0, float c1,
                                     float ih, float ih840, bool top_fs)
{
#define A8(k) a[(long long)(k) * st]
    if (j >= 4 && j <= n - 4)
        return w[0] * (A8(j) - A8(j - 1)) + w[1] * (A8(j + 1) - A8(j - 2)) + w[2] * (A8(j + 2) - A8(j - 3)) +
               w[3] * (A8(j + 3) - A8(j - 4));
    if (top_fs && j == 0) return (3675.f * A8(0) - 1225.f * A8(1) + 441.f * A8(2) - 75.f * A8(3)) * ih840;
    if (top_fs && j == 1) return (-1085.f * A8(0) + 1015.f * A8(1) - 63.f * A8(2) + 5.f * A8(3)) * ih840;
    if (j >= 2 && j <= n - 2) return c0 * (A8(j) - A8(j - 1)) + c1 * (A8(j + 1) - A8(j - 2));
    if (j == 1) return ih * (A8(1) - A8(0));
    if (j == n - 1) return ih * (A8(n - 1) - A8(n - 2));
    return 0.f;
}

// D- at cell i from positions a[0..n].
__device__ __forceinline__ float d8m(const float* a, long long st, int n, int i, const float* w, float c0, float c1,
                                     float ih, float ih24, bool top_fs)
{
    if (i >= 3 && i <= n - 4)
        return w[0] * (A8(i + 1) - A8(i)) + w[1] * (A8(i + 2) - A8(i - 1)) + w[2] * (A8(i + 3) - A8(i - 2)) +
               w[3] * (A8(i + 4) - A8(i - 3));
    if (top_fs && i == 0) return (-22.f * A8(0) + 17.f * A8(1) + 9.f * A8(2) - 5.f * A8(3) + A8(4)) * ih24;
    if (i >= 1 && i <= n - 2) return c0 * (A8(i + 1) - A8(i)) + c1 * (A8(i + 2) - A8(i - 1));
    if (i == 0) return (A8(1) - A8(0)) * ih;
    return (A8(n) - A8(n - 1)) * ih;
#undef A8
}

// Buffers of the 8th-order passes, each in the field layout (origin-based,
// row pitch ld, fstride floats per shot): u at [row][j] (j = 0..pnx), v at
// [kv][c] (kv = 0..pnz), and for the backward their adjoint counterparts
// and the rebuild's interior u / v.
struct Step8 {
    float* U;     // forward u / adjoint ubar
    float* V;     // forward v / adjoint vbar
    float* U2;    // rebuild: interior u of p^{m-1}
    float* V2;    // rebuild: interior v of p^{m-1}
};

// One receiver cell of one shot for the backward injection: the residuals of
// its receivers, syn offsets [first, first + count) of the grouped list, are
// summed in that order.
struct alignas(16) RecCell8 {
    int slot, first, count, pad;
    long long foff;          // row * ld + col
};

template <int NS>
__device__ __forceinline__ void save_strip_w(const StepParams& P, const ShotDev& sd, int row, int c, float val, int t)
{
    const Geo& g = P.g;
    const int iz = row - g.z0p, ix = c - g.x0p;
    if (iz < 0 || iz >= g.nz || ix < 0 || ix >= g.nx) return;
    const int slot = t - P.ring_t0;
    if ((unsigned)slot >= (unsigned)P.ring_slots) return;
    float* ring = P.ring + sd.ring_off + (long long)slot * P.strip_len;
    if (iz < NS) ring[iz * g.nx + ix] = val;
    if (iz >= g.nz - NS) ring[(NS + g.nz - 1 - iz) * g.nx + ix] = val;
    float* lr = ring + 2 * NS * g.nx;
    if (ix < NS) lr[ix * g.nz + iz] = val;
    if (ix >= g.nx - NS) lr[(NS + g.nx - 1 - ix) * g.nz + iz] = val;
}

template <int NS>
__device__ __forceinline__ float load_strip_w(const StepParams& P, const ShotDev& sd, int iz, int ix, int t)
{
    const Geo& g = P.g;
    const float* ring = P.ring + sd.ring_off + (long long)(t - P.ring_t0) * P.strip_len;
    if (iz < NS) return ring[iz * g.nx + ix];
    if (iz >= g.nz - NS) return ring[(NS + g.nz - 1 - iz) * g.nx + ix];
    const float* lr = ring + 2 * NS * g.nx;
    if (ix < NS) return lr[ix * g.nz + iz];
    return lr[(NS + g.nx - 1 - ix) * g.nz + iz];
}

// CPML psi update of one site (the reference's psi = b psi + a d; d += psi).
__device__ __forceinline__ float psi_fwd(const PsiSite& t, const float* psr, float* psw, const float* a0,
                                         const float* b0, const float* a1, const float* b1, float d)
{
    if (t.idx < 0) return d;
    const float ps = (t.side ? b1 : b0)[t.node] * psr[t.idx] + (t.side ? a1 : a0)[t.node] * d;
    psw[t.idx] = ps;
    return d + ps;
}

// Transposed psi of one site with carried cotangent c: t = y + c,
// ybar' = y + a t, c' = b t.  write: this thread owns the site's update.
__device__ __forceinline__ float psi_adj(const PsiSite& t, const float* psr, float* psw, const float* a0,
                                         const float* b0, const float* a1, const float* b1, float y, bool write)
{
    if (t.idx < 0) return y;
    const float tt = y + psr[t.idx];
    if (write) psw[t.idx] = (t.side ? b1 : b0)[t.node] * tt;
    return y + (t.side ? a1 : a0)[t.node] * tt;
}

#define FWI8_PML                                                                                         \
    const int n2 = 2 * P.g.npml + 1;                                                                       \
    const float* a0x = P.pmlc;          const float* b0x = a0x + n2;                                       \
    const float* a1x = a0x + 2 * n2;    const float* b1x = a0x + 3 * n2;                                   \
    const float* a0z = a0x + 4 * n2;    const float* b0z = a0x + 5 * n2;                                   \
    const float* a1z = a0x + 6 * n2;    const float* b1z = a0x + 7 * n2;

// The 8th-order passes run back to back on one stream, and on the small grids
// they serve each pass is short, so the gap between launches is a large part of
// a step.  They are launched as programmatic dependent launches: a pass may be
// scheduled while the previous one finishes, waits here for that pass to
// complete (its writes then visible) before it touches global memory, and at
// once lets the next pass be scheduled in turn.  Without a programmatic
// prerequisite (the first pass of a phase) the wait returns at once.
__device__ __forceinline__ void pdl_begin()
{
#ifndef FWI_CPU_EMU
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
#endif
}

// Forward, pass 1: u at positions (row, j), j = 0..pnx, and v at (kv, c),
// kv = 0..pnz, of p^it, each with its CPML psi.
__global__ void __launch_bounds__(256) k8_uv(const StepParams P, Step8 B)
{
    pdl_begin();
    const Geo& g = P.g;
    const Coef& cf = P.c;
    const int j = blockIdx.x * blockDim.x + threadIdx.x, r = blockIdx.y * blockDim.y + threadIdx.y;
    const int s = blockIdx.z + P.shot_base;
    if (j > g.pnx || r > g.pnz) return;
    if (P.step >= P.shots[s].nt) return;
    FWI8_PML
    const long long so = (long long)s * g.fstride;
    const float* p = P.pcur + so;
    const float* psr = P.psr + (long long)s * P.pl.stride;
    float* psw = P.psw + (long long)s * P.pl.stride;
    if (r < g.pnz) {
        float u = d8p(p + (long long)r * g.ld, 1, g.pnx, j, cf.w8x, cf.c0x, cf.c1x, cf.ix, 0.f, false);
        u = psi_fwd(psi_u(P, r, j), psr, psw, a0x, b0x, a1x, b1x, u);
        B.U[so + (long long)r * g.ld + j] = u;
    }
    if (j < g.pnx) {
        float v = d8p(p + j, g.ld, g.pnz, r, cf.w8z, cf.c0z, cf.c1z, cf.iz, cf.iz840, g.fs != 0);
        v = psi_fwd(psi_v(P, r, j), psr, psw, a0z, b0z, a1z, b1z, v);
        B.V[so + (long long)r * g.ld + j] = v;
    }
}

// Forward, pass 2: ux, vz with psi, leapfrog in place over p^{it-1}, source,
// strips of p^{it+1}.
__global__ void __launch_bounds__(256) k8_fwd(const StepParams P, Step8 B)
{
    pdl_begin();
    const Geo& g = P.g;
    const Coef& cf = P.c;
    const int c = blockIdx.x * blockDim.x + threadIdx.x, r = blockIdx.y * blockDim.y + threadIdx.y;
    const int s = blockIdx.z + P.shot_base;
    if (c >= g.pnx || r >= g.pnz) return;
    const ShotDev sd = P.shots[s];
    if (P.step >= sd.nt) return;
    FWI8_PML
    const long long so = (long long)s * g.fstride, o = so + (long long)r * g.ld + c;
    const float* psr = P.psr + (long long)s * P.pl.stride;
    float* psw = P.psw + (long long)s * P.pl.stride;
    float ux = d8m(B.U + so + (long long)r * g.ld, 1, g.pnx, c, cf.w8x, cf.c0x, cf.c1x, cf.ix, 0.f, false);
    ux = psi_fwd(psi_ux(P, r, c), psr, psw, a0x, b0x, a1x, b1x, ux);
    float vz = d8m(B.V + so + c, g.ld, g.pnz, r, cf.w8z, cf.c0z, cf.c1z, cf.iz, cf.iz24, g.fs != 0);
    vz = psi_fwd(psi_vz(P, r, c), psr, psw, a0z, b0z, a1z, b1z, vz);
    const float kk = P.K[(long long)r * g.ld + c];
    float pn = fmaf(kk, ux + vz, fmaf(2.f, P.pcur[o], -P.pold[o]));
    if (r == sd.src_r && c == sd.src_c) pn += P.wav[sd.wav_off + P.step] * cf.iarea * kk;
    P.pold[o] = pn;
    save_strip_w<NSTRIP8>(P, sd, r, c, pn, P.step);
}

// Backward, pass 1 (adjoint of b^{m+1} = y):
//   ubar(row, j) = psi_u^T( sum_i w8m(i, j) rx(i) ),  rx = psi_ux^T(y) of the row,
//   vbar(kv, c)  = psi_v^T( sum_k w8m(k, kv) rz(k) ), rz = psi_vz^T(y) of the column;
// the thread of position j (kv) also owns the psi update of cell j (kv).
// It also forms the rebuild's interior u / v of p^{m-1} on the physical grid.
__global__ void __launch_bounds__(256) k8_adj_uv(const StepParams P, Step8 B)
{
    pdl_begin();
    const Geo& g = P.g;
    const Coef& cf = P.c;
    const int j = blockIdx.x * blockDim.x + threadIdx.x, r = blockIdx.y * blockDim.y + threadIdx.y;
    const int s = blockIdx.z + P.shot_base;
    if (j > g.pnx || r > g.pnz) return;
    if (P.step > P.shots[s].nt) return;
    FWI8_PML
    const long long so = (long long)s * g.fstride;
    const float* y = P.bcur + so;
    const float* psr = P.psr + (long long)s * P.pl.stride;
    float* psw = P.psw + (long long)s * P.pl.stride;
    const int np = g.npml;
    // Away from the edges and the CPML every cell the gathers read is an
    // 8th-order cell without psi: ubar(j) = sum_k w_k (y[j-k] - y[j+k-1]), the
    // same weights as w8m, without evaluating them term by term.
    const bool fast_x = j - 4 >= max(np, 3) && j + 3 <= min(g.pnx - np - 1, g.pnx - 4);
    const bool fast_z = r - 4 >= 3 && r + 3 <= g.pnz - 4 && r + 3 < g.pnz - np - 1 && (g.fs || r - 4 > np);
    if (r < g.pnz && fast_x) {
        const float* a = y + (long long)r * g.ld;
        B.U[so + (long long)r * g.ld + j] = cf.w8x[0] * (a[j - 1] - a[j]) + cf.w8x[1] * (a[j - 2] - a[j + 1]) +
                                            cf.w8x[2] * (a[j - 3] - a[j + 2]) + cf.w8x[3] * (a[j - 4] - a[j + 3]);
    } else if (r < g.pnz) {
        float acc = 0.f;
        for (int i = j - 4; i <= j + 3; ++i) {
            const float wgt = w8m(i, j, g.pnx, cf.w8x, cf.c0x, cf.c1x, cf.ix, 0.f, false);
            if (wgt == 0.f) continue;
            const float rx = psi_adj(psi_ux(P, r, i), psr, psw, a0x, b0x, a1x, b1x, y[(long long)r * g.ld + i], false);
            acc = fmaf(wgt, rx, acc);
        }
        if (j < g.pnx)                    // this thread owns the psi update of cell j
            psi_adj(psi_ux(P, r, j), psr, psw, a0x, b0x, a1x, b1x, y[(long long)r * g.ld + j], true);
        B.U[so + (long long)r * g.ld + j] = psi_adj(psi_u(P, r, j), psr, psw, a0x, b0x, a1x, b1x, acc, true);
    }
    if (j < g.pnx && fast_z) {
        const float* a = y + j;
        const long long L = g.ld;
        B.V[so + (long long)r * g.ld + j] =
            cf.w8z[0] * (a[(r - 1) * L] - a[r * L]) + cf.w8z[1] * (a[(r - 2) * L] - a[(r + 1) * L]) +
            cf.w8z[2] * (a[(r - 3) * L] - a[(r + 2) * L]) + cf.w8z[3] * (a[(r - 4) * L] - a[(r + 3) * L]);
    } else if (j < g.pnx) {
        float acc = 0.f;
        for (int k = r - 4; k <= r + 3; ++k) {
            const float wgt = w8m(k, r, g.pnz, cf.w8z, cf.c0z, cf.c1z, cf.iz, cf.iz24, g.fs != 0);
            if (wgt == 0.f) continue;
            const float rz = psi_adj(psi_vz(P, k, j), psr, psw, a0z, b0z, a1z, b1z, y[(long long)k * g.ld + j], false);
            acc = fmaf(wgt, rz, acc);
        }
        if (r < g.pnz)
            psi_adj(psi_vz(P, r, j), psr, psw, a0z, b0z, a1z, b1z, y[(long long)r * g.ld + j], true);
        B.V[so + (long long)r * g.ld + j] = psi_adj(psi_v(P, r, j), psr, psw, a0z, b0z, a1z, b1z, acc, true);
    }
    // the rebuild's interior operator: u at physical positions [4, nx-4] of
    // rows [7, nz-7), v at physical positions [4, nz-4] of columns [7, nx-7)
    const int jp = j - g.x0p, rp = r - g.z0p;
    const float* p = P.pcur + so;
    if (rp >= 7 && rp < g.nz - 7 && jp >= 4 && jp <= g.nx - 4) {
        const float* a = p + (long long)r * g.ld;
        B.U2[so + (long long)r * g.ld + j] = cf.w8x[0] * (a[j] - a[j - 1]) + cf.w8x[1] * (a[j + 1] - a[j - 2]) +
                                             cf.w8x[2] * (a[j + 2] - a[j - 3]) + cf.w8x[3] * (a[j + 3] - a[j - 4]);
    }
    if (jp >= 7 && jp < g.nx - 7 && rp >= 4 && rp <= g.nz - 4) {
        const float* a = p + j;
        const long long L = g.ld;
        B.V2[so + (long long)r * g.ld + j] =
            cf.w8z[0] * (a[r * L] - a[(r - 1) * L]) + cf.w8z[1] * (a[(r + 1) * L] - a[(r - 2) * L]) +
            cf.w8z[2] * (a[(r + 2) * L] - a[(r - 3) * L]) + cf.w8z[3] * (a[(r + 3) * L] - a[(r - 4) * L]);
    }
}

// Backward, pass 2: pbar(c) = sum_j w8p(j, c) ubar(j) + sum_kv w8p(kv, r) vbar(kv),
// b^m = 2 b^{m+1} - b^{m+2} + K pbar in place over b^{m+2}.
__global__ void __launch_bounds__(256) k8_adj(const StepParams P, Step8 B)
{
    pdl_begin();
    const Geo& g = P.g;
    const Coef& cf = P.c;
    const int c = blockIdx.x * blockDim.x + threadIdx.x, r = blockIdx.y * blockDim.y + threadIdx.y;
    const int s = blockIdx.z + P.shot_base;
    if (c >= g.pnx || r >= g.pnz) return;
    if (P.step > P.shots[s].nt) return;
    const long long so = (long long)s * g.fstride, o = so + (long long)r * g.ld + c;
    float pbar = 0.f;
    // where every position read is an 8th-order one (c in [7, pnx-8]):
    // sum_k w_k (ubar[c-k+1] - ubar[c+k]), the weights of w8p
    if (c >= 7 && c <= g.pnx - 8) {
        const float* u = B.U + so + (long long)r * g.ld;
        pbar = cf.w8x[0] * (u[c] - u[c + 1]) + cf.w8x[1] * (u[c - 1] - u[c + 2]) + cf.w8x[2] * (u[c - 2] - u[c + 3]) +
               cf.w8x[3] * (u[c - 3] - u[c + 4]);
    } else {
        for (int j = c - 3; j <= c + 4; ++j) {
            const float wgt = w8p(j, c, g.pnx, cf.w8x, cf.c0x, cf.c1x, cf.ix, 0.f, false);
            if (wgt != 0.f) pbar = fmaf(wgt, B.U[so + (long long)r * g.ld + j], pbar);
        }
    }
    if (r >= 7 && r <= g.pnz - 8) {
        const float* v = B.V + so + c;
        const long long L = g.ld;
        pbar += cf.w8z[0] * (v[r * L] - v[(r + 1) * L]) + cf.w8z[1] * (v[(r - 1) * L] - v[(r + 2) * L]) +
                cf.w8z[2] * (v[(r - 2) * L] - v[(r + 3) * L]) + cf.w8z[3] * (v[(r - 3) * L] - v[(r + 4) * L]);
    } else {
        for (int kv = r - 3; kv <= r + 4; ++kv) {
            const float wgt = w8p(kv, r, g.pnz, cf.w8z, cf.c0z, cf.c1z, cf.iz, cf.iz840, g.fs != 0);
            if (wgt != 0.f) pbar = fmaf(wgt, B.V[so + (long long)kv * g.ld + c], pbar);
        }
    }
    const float kk = P.K[(long long)r * g.ld + c];
    P.bold[o] = fmaf(kk, pbar, fmaf(2.f, P.bcur[o], -P.bold[o]));
}

// Backward, receivers: b^m += K sum_r res[r][k] at each receiver cell of the
// launched shots, one thread per cell, receivers in input order
// (m - 1 = k jump).
__global__ void k8_inject(const StepParams P, const RecCell8* __restrict__ cells, const long long* __restrict__ syn_base,
                          int ncell, int k)
{
    pdl_begin();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ncell) return;
    const RecCell8 rc = cells[i];
    if (P.step > P.shots[rc.slot].nt) return;
    float sum = 0.f;
    for (int q = 0; q < rc.count; ++q) sum += P.res[syn_base[rc.first + q] + k];
    const long long o = (long long)rc.slot * P.g.fstride + rc.foff;
    P.bold[o] = fmaf(P.K[rc.foff], sum, P.bold[o]);
}

// Backward, pass 3 on the physical grid: p^{m-2} over p^m (the 8th-order
// interior operator of p^{m-1} plus the source inside the 7 outer
// rows/columns; the strips on them) and the imaging g += b^m (L p^{m-1} + f)
// ((p^m - 2 p^{m-1} + p^{m-2}) / K on the strips).
__global__ void __launch_bounds__(256) k8_rebuild(const StepParams P, Step8 B)
{
    pdl_begin();
    const Geo& g = P.g;
    const Coef& cf = P.c;
    const int ix = blockIdx.x * blockDim.x + threadIdx.x, iz = blockIdx.y * blockDim.y + threadIdx.y;
    const int s = blockIdx.z + P.shot_base;
    if (ix >= g.nx || iz >= g.nz) return;
    const ShotDev sd = P.shots[s];
    const int m = P.step;
    if (m > sd.nt) return;
    const int r = iz + g.z0p, c = ix + g.x0p;
    const long long so = (long long)s * g.fstride, lo = (long long)r * g.ld + c, o = so + lo;
    const float kk = P.K[lo];
    const float pm = P.pold[o], p1 = P.pcur[o];
    float pn, lp;
    if (iz >= NSTRIP8 && iz < g.nz - NSTRIP8 && ix >= NSTRIP8 && ix < g.nx - NSTRIP8) {
        const float* u = B.U2 + so + (long long)r * g.ld;
        const float* v = B.V2 + so + c;
        const long long L = g.ld;
        const float ux = cf.w8x[0] * (u[c + 1] - u[c]) + cf.w8x[1] * (u[c + 2] - u[c - 1]) +
                         cf.w8x[2] * (u[c + 3] - u[c - 2]) + cf.w8x[3] * (u[c + 4] - u[c - 3]);
        const float vz = cf.w8z[0] * (v[(r + 1) * L] - v[r * L]) + cf.w8z[1] * (v[(r + 2) * L] - v[(r - 1) * L]) +
                         cf.w8z[2] * (v[(r + 3) * L] - v[(r - 2) * L]) + cf.w8z[3] * (v[(r + 4) * L] - v[(r - 3) * L]);
        const float w = ux + vz;
        pn = fmaf(kk, w, fmaf(2.f, p1, -pm));
        lp = w;
        if (r == sd.src_r && c == sd.src_c) {
            const float f = P.wav[sd.wav_off + m - 1] * cf.iarea;
            pn += f * kk;
            lp += f;
        }
    } else {
        pn = m - 3 >= 0 ? load_strip_w<NSTRIP8>(P, sd, iz, ix, m - 3) : 0.f;
        lp = ((pm - 2.f * p1) + pn) / kk;
    }
    P.pold[o] = pn;
    P.gacc[o] = fmaf(P.bold[o], lp, P.gacc[o]);
}

#undef FWI8_PML

}  // namespace fwi
