// fwi_kernels.cuh -- sm_103a kernels of the FWI gradient hot path.
//
// One launch advances every active shot of the batch by one time step
// (grid.z = shot slot).  A thread block owns a TZ x TX tile of the padded
// grid of one shot; the pressure tile and its halo are staged in shared
// memory once, the x-direction intermediate (u, the staggered d/dx) goes
// through shared memory, and the z-direction chain (v = d/dz, vz) stays in
// registers along each thread's column segment.  u, v, ux and vz of the
// reference (fwi_2d.c:761-864) never reach HBM; the leapfrog update
// (time_integral, fwi_2d.c:866-880), source injection, receiver sampling and
// the boundary-strip save (write_bdr, fwi_2d.c:882-917) are fused into the
// epilogue.  Forward HBM traffic per cell-step: read p^it, read+write
// p^{it-1} -> p^{it+1} in place, read K (shared by all shots, L2-resident).
//
// Tiles that touch a grid edge (one-sided/edge stencils) or a CPML layer
// (psi recursions) take the GENERAL path with per-position formulas; all
// other tiles take the branch-free interior path.  The choice is uniform per
// block.
//
// The backward kernel fuses, per cell and step m = nt .. 1,
//   * the exact adjoint b^m = 2 b^{m+1} - b^{m+2} + K (L^T b^{m+1} + r^m) on
//     the padded grid (L^T is the transpose of the CPML operator, including
//     the adjoint of its psi recursions),
//   * the source-field rebuild p^{m-2} = 2 p^{m-1} - p^m + K L p^{m-1} + s^{m-1}
//     on the physical interior (a_lap_opt_2d, fwi_2d.c:722-759), with the
//     three outer rows/columns restored from the strip ring (read_bdr,
//     fwi_2d.c:919-960),
//   * the imaging condition g += b^m (L p^{m-1} + f^{m-1}).
#pragma once
#ifdef FWI_CPU_EMU
#include "cpu_emu.h"
#else
#include <cuda_runtime.h>
#include <cuda_fp16.h>
#include <cuda_bf16.h>
#include "cpu_emu.h"
#endif
#include <stdint.h>
#include <cstdio>

namespace fwi {

// Self-checking diagnostics build (FWI_SELF_CHECK, never the product build):
// every shared-memory index goes through SIDX and every global pointer that
// is dereferenced through GP.  A shared index outside its array or a global
// access outside the registered allocations (or misaligned for its type) is
// recorded once in g_check (site = source line) and redirected to a valid
// dummy location, so a checked kernel cannot fault.  Product builds compile
// both macros to the plain expression.
struct DbgRanges {
    unsigned long long lo[24], hi[24];
    int n;
};
struct CheckRec {
    int bad, site;
    long long idx, lim;
    int bx, by, bz, tx, ty;
};
#ifdef FWI_SELF_CHECK
__device__ DbgRanges g_dbg;
__device__ CheckRec g_check;
__device__ __align__(16) float g_sink[16];
__device__ inline void check_record(int site, long long idx, long long lim)
{
    if (atomicCAS(&g_check.bad, 0, 1) == 0) {
        g_check.site = site;
        g_check.idx = idx;
        g_check.lim = lim;
        g_check.bx = blockIdx.x; g_check.by = blockIdx.y; g_check.bz = blockIdx.z;
        g_check.tx = threadIdx.x; g_check.ty = threadIdx.y;
    }
}
__device__ inline int sidx(int i, int n, int site)
{
    if ((unsigned)i < (unsigned)n) return i;
    check_record(site, i, n);
    return 0;
}
template <class T>
__device__ inline T* gptr(T* p, int site)
{
    const unsigned long long a = (unsigned long long)p;
    const unsigned long long al = sizeof(T) >= 16 ? 16 : sizeof(T);
    bool in = false;
    for (int i = 0; i < g_dbg.n; ++i)
        if (a >= g_dbg.lo[i] && a + sizeof(T) <= g_dbg.hi[i]) { in = true; break; }
    if (in && a % al == 0) return p;
    check_record(site, (long long)a, in ? -2 : -1);   // lim -1: outside every allocation, -2: misaligned
    return reinterpret_cast<T*>(g_sink);
}
#define SIDX(i, n) ::fwi::sidx((i), (n), __LINE__)
#define GP(p) ::fwi::gptr((p), __LINE__)
#else
#define SIDX(i, n) (i)
#define GP(p) (p)
#endif

// Block timeline diagnostics build (FWI_TIMELINE, never the product build):
// thread (0, 0) of every block of the stencil kernels records %globaltimer
// when the block starts a work item and, after a barrier, when it ends it,
// at one time step (g_tl_step), into g_tl[class][item][start, end].  Classes:
// 0 interior backward, 1 z-general, 2 x-general, 3 corner backward tiles,
// 4 interior forward, 5-7 the forward general classes.  The engine arms it
// from the environment (FWI_TIMELINE_STEP, FWI_TIMELINE_OUT) and writes the
// buffer out when the context is destroyed; the product build compiles
// FWI_TL to nothing.
constexpr long long TL_ITEMS = 1LL << 16;        // items recorded per class
#ifdef FWI_TIMELINE
__device__ unsigned long long* g_tl = nullptr;
__device__ int g_tl_step = -1;
__device__ __forceinline__ void tl_stamp(int step, int cls, long long item, int end)
{
    if (!g_tl || step != g_tl_step || threadIdx.x != 0 || threadIdx.y != 0 || item < 0 || item >= TL_ITEMS) return;
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    g_tl[((long long)cls * TL_ITEMS + item) * 2 + end] = t;
}
#define FWI_TL(step, cls, item, end) tl_stamp((step), (cls), (item), (end))
#define FWI_TL_END(step, cls, item) do { __syncthreads(); tl_stamp((step), (cls), (item), 1); } while (0)
#else
#define FWI_TL(step, cls, item, end) ((void)0)
#define FWI_TL_END(step, cls, item) ((void)0)
#endif
// Timeline class of a general tile class (GX, GZ): base + 1 z-general, + 2 x-general, + 3 corners.
__host__ __device__ constexpr int tl_class(bool gx, bool gz, int base) { return base + (gx && gz ? 3 : gx ? 2 : 1); }

constexpr int TX = 64;             // tile width  (cells)
constexpr int TZ = 32;             // tile height (cells)
constexpr int BX = 32;             // threads in x
constexpr int BY = 8;              // threads in z
constexpr int NTH = BX * BY;
constexpr int R = TZ / BY;         // rows per thread
constexpr int CX = TX / BX;        // columns per thread
constexpr int HX = 4;              // x halo staged (>= 3, multiple of 4 for float4)
constexpr int HZ = 3;              // z halo staged
constexpr int SPW = TX + 2 * HX;   // staged tile width  (72)
constexpr int SPH = TZ + 2 * HZ;   // staged tile height (38)
constexpr int UW = TX + 3;         // u positions x0-1 .. x0+TX+1
constexpr int UWP = TX + 4;        // u row pitch
constexpr int RXW = TX + 6;        // adjoint x-stage positions x0-3 .. x0+TX+2
constexpr int RXP = TX + 8;
constexpr int MZ = 4;              // zero margin rows above the first tile's halo and below the last tile
constexpr int NSTRIP = 3;          // 2*mm-1 saved rows/columns per side (fwi_sys.h:7, mm = 2)

struct Geo {
    int nx, nz;        // physical grid
    int pnx, pnz;      // padded grid (fwi_2d.c:154-165)
    int npml, fs;
    int x0p, z0p;      // physical origin in padded coordinates
    int ld;            // row pitch of every field array (floats)
    int ntx, ntz;      // tiles per shot
    int xoff;          // padded column of tile column 0 (<= 0): the tile grid starts where the
                       // first interior tile can start, so general tiles hold few columns
    int zoff;          // padded row of tile row 0 (<= 0, a multiple of R), the same for rows
    long long fstride; // floats between consecutive shots in a field array
};

struct Coef {
    float c0x, c1x, ix, c0z, c1z, iz, iz840, iz24;   // fwi_2d.c:304-314
    float iarea;                                     // fwi_2d.c:216
    float wx1, wx2, wx3;                             // dxx7 weights (from c0x, c1x)
    float w8x[4], w8z[4];                            // 8th-order staggered weights / h (fd_order 8)
};

// The x part of the plain operator, ux(c) = c0 (u(c+1) - u(c)) + c1 (u(c+2) -
// u(c-1)) with u(j) = c0 (p[j] - p[j-1]) + c1 (p[j+1] - p[j-2])
// (fwi_2d.c:775-784, 822-827), as one symmetric stencil of p[c-3 .. c+3]
// with weights w1 = c0^2 - 2 c0 c1, w2 = 2 c0 c1, w3 = c1^2 for the
// neighbours at distance 1, 2, 3 and -2 (w1 + w2 + w3) for the cell.  The
// weights sum to zero, so it is evaluated on differences from the cell,
// d_k = (p[c+k] - p[c]) + (p[c-k] - p[c]), which keeps the accuracy of the
// two-stage form on smooth fields.  The adjoint x part of an interior tile
// is the same stencil of b.  st[i] is the staged value at the cell.
__device__ __forceinline__ float dxx7(const float* st, int i, const Coef& cf)
{
    [[maybe_unused]] constexpr int NS = SPH * SPW;
    const float p0 = st[SIDX(i, NS)];
    const float d1 = (st[SIDX(i + 1, NS)] - p0) + (st[SIDX(i - 1, NS)] - p0);
    const float d2 = (st[SIDX(i + 2, NS)] - p0) + (st[SIDX(i - 2, NS)] - p0);
    const float d3 = (st[SIDX(i + 3, NS)] - p0) + (st[SIDX(i - 3, NS)] - p0);
    return cf.wx1 * d1 + cf.wx2 * d2 + cf.wx3 * d3;
}

// psi arrays of one shot, in the order u0,u1,v0,v1,ux0,ux1,vz0,vz1
// (pml_profile, header.h:97; shapes fwi_2d.c:288-296).
struct PsiLayout {
    long long stride;  // floats per shot
    int u0, u1, v0, v1, ux0, ux1, vz0, vz1;
};

// Device-side records are padded to multiples of 16 bytes and 16-byte
// aligned, so that every array element can be read with vector loads.
struct alignas(16) ShotDev {
    int nt, nt0, nr;
    int src_r, src_c;        // source cell, padded coordinates
    int wav_off;             // offset of the wavelet in the wavelet pool
    int rtile_off;           // offset of this shot's per-tile receiver CSR
    int pad;
    long long syn_off;       // offset of the shot's traces in syn/res/obs
    long long ring_off;      // offset of the shot's strip ring
};

// One receiver, for sampling syn[r][k] = p^{k*jump+1}(receiver).
struct alignas(16) RecSample {
    int slot, pad0;
    long long foff;          // row * ld + col of the receiver cell
    long long syn_base;      // syn_off + r * nt0
    long long pad1;
};

// One receiver for the backward injection, grouped by tile.
struct alignas(16) RecDev {
    int cell;                // (row - z0) * TX + (col - x0) inside its tile at (z0, x0)
    int pad;
    long long syn_base;      // syn_off + r * nt0
};

struct RecParams {
    Geo g;
    const ShotDev* shots;
    const RecSample* recs;   // sampling
    float* field;            // p^{it+1}
    float* syn;
    int lo, hi;              // receiver range of this launch
    int step, jump;
};

// A CUtensorMap (128 bytes, 64-byte aligned) encoded on the host for one
// field half: dims (ld, rows_alloc, shots) of floats, box SPW x SPH x 1.
struct alignas(64) TensorMap {
    unsigned long long w[16];
};

struct StepParams {
    Geo g;
    Coef c;
    const float* K;          // padded K = v^2 dt^2 (one copy for all shots)
    const float* pcur;       // p^it (forward) / p^{m-1} (backward)
    float* pold;             // p^{it-1} -> p^{it+1} / p^m -> p^{m-2}, in place
    const float* bcur;       // b^{m+1}
    float* bold;             // b^{m+2} -> b^m, in place
    float* gacc;             // imaging accumulator, field layout, per shot
    const float* psr;        // psi (or adjoint psi) read at this step
    float* psw;              // psi written at this step
    const float* pmlc;       // a0x b0x a1x b1x a0z b0z a1z b1z, 2*npml+1 each
    PsiLayout pl;
    const ShotDev* shots;
    const int2* gen_tiles;   // tiles of the general path (x tile, z tile)
    int fast_tx0, fast_tz0;  // interior tile rectangle [fast_tx0, fast_tx1) x [fast_tz0, fast_tz1)
    int fast_tx1, fast_tz1;
    int gen_arith;           // general tiles follow from the rectangle (gen_tile_at), no list read
    int gen_n;               // tiles of the general class launched
    int gen_shots;           // shots of the launch (slots shot_base ..)
    const RecDev* recs;      // backward: receivers grouped by tile
    const int* rtile;        // backward: per-tile CSR of recs
    const float* wav;
    float* syn;              // forward: sampled traces
    const float* res;        // backward: adjoint sources
    float* ring;             // boundary strips
    int strip_len;
    int ring_t0;             // the strip of p^{t+1} (saved at step t) sits in ring slot t - ring_t0
    int ring_slots;          // slots per shot; strips whose slot falls outside are not saved
    int step;                // forward: it; backward: m
    int jump;
    int shot_base;           // slot of blockIdx.z == 0 (non-zero only when shots run one by one)
    int* err;                // set to 1 by a block whose tile copy did not complete (bounded wait)
    TensorMap tm_pcur;       // pcur's field half (interior tiles stage it with TMA)
    TensorMap tm_bcur;       // bcur's field half (backward)
};

// A tile takes the general path when its cells or their stencil halo touch a
// grid edge (edge and one-sided formulas), a CPML layer (psi recursions) or
// the boundary strips.  The test separates into x and z, so the interior
// tiles form a rectangle.
//
// The same tests apply to any window of w columns (h rows): a window whose
// test is false lies, with the stencil reach of its outputs (3 cells), inside
// the region where every formula is the plain interior one.  Inside a
// general tile, warps use them to take the plain formulas for their own rows
// (z window of R rows) or column half (x window of BX columns).
__host__ __device__ inline bool x_window_general(const Geo& g, int x0, int w)
{
    const int np = g.npml;
    return x0 < 8 || x0 + w + 8 > g.pnx || x0 - 4 <= np || x0 + w + 4 >= g.pnx - np;
}
__host__ __device__ inline bool z_window_general(const Geo& g, int z0, int h)
{
    const int np = g.npml;
    return z0 < 8 || z0 + h + 8 > g.pnz || z0 + h + 4 >= g.pnz - np || (!g.fs && z0 - 4 <= np);
}
__host__ __device__ inline bool tile_x_general(const Geo& g, int x0) { return x_window_general(g, x0, TX); }
// The w positions from j0 all lie outside [lo, hi]: in the x stages of the
// tiles at the grid's ends, such windows have no psi site and a zero result.
__device__ __forceinline__ bool x_window_outside(int j0, int w, int lo, int hi) { return j0 + w <= lo || j0 > hi; }
__host__ __device__ inline bool tile_z_general(const Geo& g, int z0) { return z_window_general(g, z0, TZ); }

// A z-general unit of R rows from r0 needs the grid-edge formulas (free
// surface, one-sided differences at rows 0, 1, pnz-2, pnz-1, values outside
// the grid) only near the top or bottom of the grid; elsewhere (a CPML band)
// it takes the plain differences and the psi recursions.  The margins are the
// reach of the adjoint's one-sided terms (rows r0-3 .. r0+R+2 against rows 1
// and pnz-2, and the free-surface terms of rows up to 4), which is the wider.
__device__ __forceinline__ bool z_unit_edge(const Geo& g, int r0) { return r0 < 8 || r0 + R + 4 > g.pnz; }

// Staged rows a z-only general tile reads: those of its rows inside the padded
// grid and HZ more on either side (staged row r holds grid row z0 - HZ + r).
// Its row-group units start inside the grid and every cell it writes reads
// rows within HZ of its own, so the rows outside this range (most of a tile
// above the first grid row) need not be copied.
__device__ __forceinline__ int2 z_tile_rows(const Geo& g, int z0)
{
    return make_int2(max(z0, 0) - z0, min(z0 + TZ, g.pnz) - z0 + 2 * HZ);
}

// Tile i of a general class, from the interior tile rectangle [tx0, tx1) x
// [tz0, tz1): the x-general class is the general columns (left, then right)
// of the interior rows, the z-general class the interior columns of the
// general rows (top, then bottom), the corners the general columns of the
// general rows, each row by row.  The engine checks this against its tile
// lists; it spares every general block a dependent load before its copies.
__host__ __device__ inline int2 gen_tile_at(const Geo& g, int tx0, int tx1, int tz0, int tz1, bool gx, bool gz, int i)
{
    const int ncol = gx ? g.ntx - (tx1 - tx0) : tx1 - tx0;
    const int cx = i % ncol, cz = i / ncol;
    const int tx = gx ? (cx < tx0 ? cx : cx - tx0 + tx1) : tx0 + cx;
    const int tz = gz ? (cz < tz0 ? cz : cz - tz0 + tz1) : tz0 + cz;
    return make_int2(tx, tz);
}

// Work units of the z phases of a general tile: a row group of R rows and a
// column half.  A tile with L row groups inside the padded grid has L * CX
// units, and warp ty takes units ty and ty + BY (q = 0, 1).  In a full tile
// (L == BY) that is the warp's own R rows in both halves; in a tile with few
// live groups (the free-surface band above the interior has two) the units
// spread over more warps, so the block holds its slot for a shorter time.
struct ZUnit {
    int r0l, h;        // first local row, column half
    bool live;
};
template <bool GZ>
__device__ __forceinline__ ZUnit z_unit(const Geo& g, int z0, int q)
{
    if (!GZ) return {R * (int)threadIdx.y, q, true};                       // tiles inside the grid in z
    const int lo = max(z0, 0), hi = min(z0 + TZ, g.pnz);                   // z0 and 0 are multiples of R
    const int gl0 = (lo - z0) / R, L = (hi - z0 + R - 1) / R - gl0;
    const int u = threadIdx.y + BY * q;
    if (u >= L * CX) return {0, 0, false};
    return {R * (gl0 + u % L), u / L, true};
}

// CPML psi sites.  Each returns the offset of the psi entry within one shot's
// psi block (or -1 where the position has none) and the profile node and
// side of its coefficients (side 0: a0/b0 = left/top, 1: a1/b1 = right/bottom).
// u positions j in [0, pnx] (fwi_2d.c:790-794), ux cells i in [0, pnx)
// (838-842), v positions kv in [0, pnz] (816-817; v0 mirrors v1 on top when
// free_surface == 0), vz cells (860-861).  The kernels read all psi entries
// of a phase with independent loads before they use any of them.
struct PsiSite {
    int idx, node, side;
};
__device__ __forceinline__ PsiSite psi_u(const StepParams& P, int row, int j)
{
    const int np = P.g.npml, pnx = P.g.pnx;
    if (j >= 0 && j <= np) return {P.pl.u0 + row * (np + 1) + j, 2 * j, 0};
    if (j >= pnx - np && j <= pnx) return {P.pl.u1 + row * (np + 1) + (j - (pnx - np)), 2 * (j - (pnx - np)), 1};
    return {-1, 0, 0};
}
__device__ __forceinline__ PsiSite psi_ux(const StepParams& P, int row, int i)
{
    const int np = P.g.npml, pnx = P.g.pnx;
    if (i >= 0 && i < np) return {P.pl.ux0 + row * np + i, 2 * i + 1, 0};
    if (i >= pnx - np && i < pnx) return {P.pl.ux1 + row * np + (i - (pnx - np)), 2 * (i - (pnx - np)) + 1, 1};
    return {-1, 0, 0};
}
__device__ __forceinline__ PsiSite psi_v(const StepParams& P, int kv, int c)
{
    const int np = P.g.npml, pnx = P.g.pnx, pnz = P.g.pnz;
    if (c < 0 || c >= pnx || kv < 0 || kv > pnz) return {-1, 0, 0};
    if (kv >= pnz - np) return {P.pl.v1 + (kv - (pnz - np)) * pnx + c, 2 * (kv - (pnz - np)), 1};
    if (!P.g.fs && kv <= np) return {P.pl.v0 + kv * pnx + c, 2 * kv, 0};
    return {-1, 0, 0};
}
__device__ __forceinline__ PsiSite psi_vz(const StepParams& P, int row, int c)
{
    const int np = P.g.npml, pnx = P.g.pnx, pnz = P.g.pnz;
    if (c < 0 || c >= pnx || row < 0 || row >= pnz) return {-1, 0, 0};
    if (row >= pnz - np) return {P.pl.vz1 + (row - (pnz - np)) * pnx + c, 2 * (row - (pnz - np)) + 1, 1};
    if (!P.g.fs && row < np) return {P.pl.vz0 + row * pnx + c, 2 * row + 1, 0};
    return {-1, 0, 0};
}
// psi value of a site (0 where there is none)
__device__ __forceinline__ float psi_load(const float* psr, const PsiSite& t) { return t.idx >= 0 ? __ldcg(GP(psr + t.idx)) : 0.f; }

// The psi sites of a general tile, one entry per row (z sites) or column (x
// sites) within its reach, built once per block by psi_v / psi_vz at column 0
// and psi_u / psi_ux at row 0: off is the site's offset there (-1: no site)
// and a, b its recursion coefficients.  A z site of column c is off + c (c in
// [0, pnx)); an x site of row r is off + r (np + 1) for u and off + r np for
// ux (r in [0, pnz)).  The tile bodies read one entry instead of deciding the
// site and loading its coefficients per element.
struct PsiRowSite {
    int off;
    float a, b;
    int pad;
};
struct ZSiteTab {
    PsiRowSite zvz[TZ + 6];    // vz cells, rows z0-3 .. z0+TZ+2
    PsiRowSite zv[TZ + 3];     // v positions, rows z0-1 .. z0+TZ+1
};
struct XSiteTab {
    PsiRowSite xux[RXW];       // ux cells, columns x0-3 .. x0+TX+2
    PsiRowSite xu[UW];         // u positions, columns x0-1 .. x0+TX+1
};
__device__ __forceinline__ PsiRowSite row_site(const StepParams& P, const PsiSite& t, int axis)
{
    // pmlc holds a0x b0x a1x b1x a0z b0z a1z b1z, 2 npml + 1 each
    const int n2 = 2 * P.g.npml + 1;
    if (t.idx < 0) return {-1, 0.f, 0.f, 0};
    const float* base = P.pmlc + (axis * 4 + t.side * 2) * n2;
    return {t.idx, *GP(base + t.node), *GP(base + n2 + t.node), 0};
}
// Fills the tables a tile of class (GX, GZ) at (x0, z0) reads; a barrier must
// follow before they are read.
template <bool GX, bool GZ>
__device__ __forceinline__ void fill_sites(const StepParams& P, int x0, int z0, ZSiteTab& tz, XSiteTab& tx)
{
    const int tid = threadIdx.y * BX + threadIdx.x;
    if (GZ)
        for (int i = tid; i < 2 * TZ + 9; i += NTH) {
            if (i < TZ + 6) tz.zvz[i] = row_site(P, psi_vz(P, z0 - 3 + i, 0), 1);
            else tz.zv[i - (TZ + 6)] = row_site(P, psi_v(P, z0 - 1 + (i - (TZ + 6)), 0), 1);
        }
    if (GX)
        for (int i = tid; i < RXW + UW; i += NTH) {
            if (i < RXW) tx.xux[i] = row_site(P, psi_ux(P, 0, x0 - 3 + i), 0);
            else tx.xu[i - RXW] = row_site(P, psi_u(P, 0, x0 - 1 + (i - RXW)), 0);
        }
}

// u = staggered d/dx of p at u-position j (fwi_2d.c:775-784); p[row][col]
// is sp[base + col] (base = row offset - x0 + HX, an integer, so no pointer
// leaves the array).
__device__ __forceinline__ float u_edge(const float* sp, int base, int j, int pnx, const Coef& c)
{
    #define PX(col) sp[SIDX(base + (col), SPH * SPW)]
    if (j >= 2 && j <= pnx - 2) return c.c0x * (PX(j) - PX(j - 1)) + c.c1x * (PX(j + 1) - PX(j - 2));
    if (j == 1) return c.ix * (PX(1) - PX(0));
    if (j == pnx - 1) return c.ix * (PX(pnx - 1) - PX(pnx - 2));
    #undef PX
    return 0.f;   // u[0], u[pnx] are never assigned by the reference
}

// 16-byte global -> shared copy that bypasses the registers (cp.async), so a
// thread's copies of a tile are all in flight at once.  cp_async_wait()
// completes the calling thread's copies; the barrier after it publishes the
// tile to the block.  The CPU emulation copies at once.
__device__ __forceinline__ void cp_async16(float* dst, const float4* src)
{
#ifdef FWI_CPU_EMU
    *reinterpret_cast<float4*>(dst) = *src;
#else
    const unsigned sa = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(src) : "memory");
#endif
}
__device__ __forceinline__ void cp_async_wait()
{
#ifndef FWI_CPU_EMU
    asm volatile("cp.async.wait_all;\n" ::: "memory");
#endif
}

// Tensor-memory-access (TMA) copies of staged tiles: one thread arms an
// mbarrier with the expected bytes and issues cp.async.bulk.tensor; every
// thread waits on the barrier's phase 0.  The wait is bounded: a block whose
// copy has not landed after its own TMA_WAIT_CYCLES (about half a second)
// sets *err and skips its tile, and the host reports the error and refuses
// further work on the context.  A block never gives up earlier (for example
// because another block raised the flag), so it does not leave while its own
// copy may still land in its shared memory.  Tile destinations are 128-byte
// aligned; the x coordinate x0 - xoff is a multiple of 64 floats.
constexpr long long TMA_WAIT_CYCLES = 1LL << 30;
constexpr unsigned TILE_BYTES = SPH * SPW * sizeof(float);
#ifndef FWI_CPU_EMU
__device__ __forceinline__ unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(unsigned long long* bar)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(bar)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned long long* bar, unsigned bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait0(unsigned long long* bar)
{
    unsigned ok;
    asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0;\n selp.u32 %0, 1, 0, p;\n}\n"
                 : "=r"(ok) : "r"(smem_u32(bar)) : "memory");
    return ok != 0;
}
// The tile of the field half tm whose interior starts at (z0, x0), shot s.
__device__ __forceinline__ void tma_tile(float* dst, const TensorMap* tm, const Geo& g, int x0, int z0, int s,
                                         unsigned long long* bar)
{
    const int x = x0 - g.xoff, y = z0 - g.zoff + MZ - HZ;             // allocation column and row of the box
    asm volatile("cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
                 " [%0], [%1, {%2, %3, %4}], [%5];\n"
                 ::"r"(smem_u32(dst)), "l"(tm), "r"(x), "r"(y), "r"(s), "r"(smem_u32(bar)) : "memory");
}
// Bounded wait for phase 0; false (and *err set) when it did not complete.
__device__ __forceinline__ bool tma_wait(unsigned long long* bar, int* err)
{
    const long long t0 = clock64();
    for (unsigned i = 1;; ++i) {
        if (mbar_try_wait0(bar)) return true;
        if ((i & 1023u) == 0 && clock64() - t0 > TMA_WAIT_CYCLES) break;
    }
    atomicExch(err, 1);
    return false;
}
#endif

// Starts copying the (TZ+2HZ) x (TX+2HX) tile of field f whose interior
// starts at (z0, x0) into shared memory in 16-byte pieces; cp_async_wait()
// and a barrier must follow before the tile is read.
// Rows r_lo .. r_hi - 1 of the staged tile only (default: all SPH rows).
__device__ __forceinline__ void stage_tile(const float* __restrict__ f, const Geo& g, int x0, int z0, float* sp,
                                           int r_lo = 0, int r_hi = SPH)
{
    const int tid = threadIdx.y * BX + threadIdx.x;
    constexpr int Q = SPW / 4;
    for (int i = r_lo * Q + tid; i < r_hi * Q; i += NTH) {
        const int r = i / Q, q = i - r * Q;
        const float4* src = reinterpret_cast<const float4*>(f + (long long)(z0 - HZ + r) * g.ld + (x0 - HX) + 4 * q);
        cp_async16(sp + SIDX(r * SPW + 4 * q, SPH * SPW), GP(src));
    }
}

__device__ __forceinline__ void save_strip(const StepParams& P, const ShotDev& sd, int row, int c, float val, int t)
{
    const Geo& g = P.g;
    const int iz = row - g.z0p, ix = c - g.x0p;
    if (iz < 0 || iz >= g.nz || ix < 0 || ix >= g.nx) return;
    const int slot = t - P.ring_t0;
    if ((unsigned)slot >= (unsigned)P.ring_slots) return;      // outside the ring of the current segment
    float* ring = P.ring + sd.ring_off + (long long)slot * P.strip_len;
    if (iz < NSTRIP) *GP(ring + iz * g.nx + ix) = val;
    if (iz >= g.nz - NSTRIP) *GP(ring + (NSTRIP + g.nz - 1 - iz) * g.nx + ix) = val;
    float* lr = ring + 2 * NSTRIP * g.nx;
    if (ix < NSTRIP) *GP(lr + ix * g.nz + iz) = val;
    if (ix >= g.nx - NSTRIP) *GP(lr + (NSTRIP + g.nx - 1 - ix) * g.nz + iz) = val;
}

__device__ __forceinline__ float load_strip(const StepParams& P, const ShotDev& sd, int iz, int ix, int t)
{
    const Geo& g = P.g;
    const float* ring = P.ring + sd.ring_off + (long long)(t - P.ring_t0) * P.strip_len;
    if (iz < NSTRIP) return *GP(ring + iz * g.nx + ix);
    if (iz >= g.nz - NSTRIP) return *GP(ring + (NSTRIP + g.nz - 1 - iz) * g.nx + ix);
    const float* lr = ring + 2 * NSTRIP * g.nx;
    if (ix < NSTRIP) return *GP(lr + ix * g.nz + iz);
    return *GP(lr + (NSTRIP + g.nx - 1 - ix) * g.nz + iz);
}

// Adjoint sources of one tile: racc[cell] = the sum of res[r][k] over the
// tile's receivers r in that cell.  The receivers of a tile, recs[rb, re),
// are sorted by cell and, within a cell, by input order; the thread that
// holds the first receiver of a cell adds up that run in order, so the sum
// is the same on every run (no atomics).  racc must be zero beforehand.
__device__ __forceinline__ void gather_residuals(const StepParams& P, int rb, int re, int k, float* racc)
{
    const int tid = threadIdx.y * BX + threadIdx.x;
    for (int q = rb + tid; q < re; q += NTH) {
        const RecDev rd = *GP(P.recs + q);
        if (q > rb && GP(P.recs + q - 1)->cell == rd.cell) continue;       // not the first of its cell
        float sum = *GP(P.res + rd.syn_base + k);
        for (int j = q + 1; j < re; ++j) {
            const RecDev rn = *GP(P.recs + j);
            if (rn.cell != rd.cell) break;
            sum += *GP(P.res + rn.syn_base + k);
        }
        racc[SIDX(rd.cell, TZ * TX)] = sum;
    }
}

// ---------------------------------------------------------------------------
// Forward step
// ---------------------------------------------------------------------------
// One forward tile.  GX / GZ select the general (edge, CPML and strip aware)
// formulas along x / z; an axis whose general flag is false takes the plain
// interior stencil, which the tile classification (tile_x_general,
// tile_z_general) guarantees to be exact there.  In tiles that reach past the
// padded grid, warps whose rows all lie beyond pnz and column halves beyond
// pnx skip their work (uniform per warp).
template <bool GX, bool GZ>
__device__ __forceinline__ void fwd_tile(const StepParams& P, const ShotDev& sd, int s, int x0, int z0,
                                         float* sp, float* su, const ZSiteTab& tbz, const XSiteTab& tbx)
{
    const Geo& g = P.g;
    const Coef& cf = P.c;
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int np = g.npml;
    const long long so = (long long)s * g.fstride;
    const float* __restrict__ psr = P.psr + (long long)s * P.pl.stride;
    float* __restrict__ psw = P.psw + (long long)s * P.pl.stride;

    // u at positions j in [x0-1, x0+TX+1], rows [z0, z0+TZ); the psi entries
    // of the x-general column halves are read first
    float pu[R][3];
    if (GX) {
        #pragma unroll
        for (int k = 0; k < R; ++k) {
            const int row = z0 + ty + BY * k;
            #pragma unroll
            for (int h = 0; h < 3; ++h) {
                const int jj = tx + BX * h;
                const bool gen = jj < UW && !(GZ && (row < 0 || row >= g.pnz)) && x_window_general(g, x0 - 1 + BX * h, BX) &&
                                 !x_window_outside(x0 - 1 + BX * h, BX, 0, g.pnx);
                const int off = gen ? tbx.xu[jj].off : -1;
                pu[k][h] = off >= 0 ? __ldcg(GP(psr + off + row * (np + 1))) : 0.f;
            }
        }
    }
    // u positions into su: x-general tiles only (elsewhere the x part is dxx7 of sp)
    #pragma unroll
    for (int k = 0; k < R; ++k) {
        if (!GX) break;
        const int rl = ty + BY * k, row = z0 + rl;
        if (GZ && (row < 0 || row >= g.pnz)) continue;                      // rows outside the grid
        const int pbase = (rl + HZ) * SPW + HX - x0;                       // + global column = sp index
        #pragma unroll
        for (int h = 0; h < 3; ++h) {
            const int jj = tx + BX * h;
            if (jj >= UW) break;
            const int j = x0 - 1 + jj;
            float u;
            if (!GX || !x_window_general(g, x0 - 1 + BX * h, BX)) {        // plain u for this column half
                const int q = pbase + j;
                u = cf.c0x * (sp[SIDX(q, SPH * SPW)] - sp[SIDX(q - 1, SPH * SPW)]) +
                    cf.c1x * (sp[SIDX(q + 1, SPH * SPW)] - sp[SIDX(q - 2, SPH * SPW)]);
            } else if (x_window_outside(x0 - 1 + BX * h, BX, 0, g.pnx)) {  // u positions are 0 .. pnx
                u = 0.f;
            } else {
                u = u_edge(sp, pbase, j, g.pnx, cf);
                const PsiRowSite e = tbx.xu[jj];                             // fwi_2d.c:790-794
                if (e.off >= 0) {
                    const float ps = e.b * pu[k][h] + e.a * u;
                    if (jj >= 1 && jj <= TX) *GP(psw + e.off + row * (np + 1)) = ps;
                    u += ps;
                }
            }
            su[SIDX(rl * UWP + jj, TZ * UWP)] = u;
        }
    }
    if (GX) __syncthreads();

    const float* __restrict__ K = P.K;
    float* __restrict__ pold = P.pold + so;
    const float amp = *GP(P.wav + sd.wav_off + P.step) * cf.iarea;
    #pragma unroll
    for (int q = 0; q < CX; ++q) {
        const ZUnit zu = z_unit<GZ>(g, z0, q);
        if (!zu.live) continue;                                            // the last phase: no barrier follows
        const int r0l = zu.r0l, r0 = z0 + r0l, h = zu.h;
        const bool gzw = GZ && z_window_general(g, r0, R);                 // this unit's rows need the z-general formulas
        const bool gze = gzw && z_unit_edge(g, r0);                        // ... and the grid-edge ones among them
        if (GX && (x0 + BX * h >= g.pnx || x0 + BX * h + BX <= 0)) continue;   // column half outside the grid
        const bool gxc = GX && x_window_general(g, x0 + BX * h, BX);        // this half needs the x-general formulas
        const int cl = tx + BX * h, c = x0 + cl;
        const bool cin = !GX || (c >= 0 && c < g.pnx);                      // z sites exist in grid columns only
        // strip cells (saved for the backward rebuild) of this unit: its rows meet the
        // first or last NSTRIP physical rows, or this column is one of the first or last
        // NSTRIP physical columns; save_strip checks each cell again
        const int izu = r0 - g.z0p, ixc = c - g.x0p;
        const bool strip_rows = gzw && ((izu < NSTRIP && izu + R > 0) || (izu + R > g.nz - NSTRIP && izu < g.nz));
        const bool strip_col = gxc && ((ixc >= 0 && ixc < NSTRIP) || (ixc >= g.nx - NSTRIP && ixc < g.nx));
        // every global operand of this column segment first: K, p^{it-1} and the psi entries
        float kq[R], po[R], pvv[R + 3], pux[R], pvz[R];
        const int xoff = gxc ? tbx.xux[cl + 3].off : -1;                     // the ux site of column c
        #pragma unroll
        for (int i = 0; i < R; ++i) {
            const int row = r0 + i;
            const bool inside = (!GZ || row < g.pnz) && (!GX || (c >= 0 && c < g.pnx));
            const long long o = (long long)row * g.ld + c;
            kq[i] = inside ? __ldg(GP(K + o)) : 0.f;
            po[i] = inside ? *GP(pold + o) : 0.f;
            pux[i] = (inside && xoff >= 0) ? __ldcg(GP(psr + xoff + row * np)) : 0.f;
            const int zoff = (gzw && inside) ? tbz.zvz[r0l + i + 3].off : -1;
            pvz[i] = zoff >= 0 ? __ldcg(GP(psr + zoff + c)) : 0.f;
        }
        #pragma unroll
        for (int k = 0; k < R + 3; ++k) {
            const int off = (gzw && cin) ? tbz.zv[r0l + k].off : -1;
            pvv[k] = off >= 0 ? __ldcg(GP(psr + off + c)) : 0.f;
        }

        float pc[R + 6];
        #pragma unroll
        for (int k = 0; k < R + 6; ++k) pc[k] = sp[SIDX((r0l + k) * SPW + HX + cl, SPH * SPW)];   // rows r0-3+k
        float vv[R + 3];                                                            // v rows r0-1+k
        #pragma unroll
        for (int k = 0; k < R + 3; ++k) {
            const int kv = r0 - 1 + k;
            float v;
            if (!gzw) {
                v = cf.c0z * (pc[k + 2] - pc[k + 1]) + cf.c1z * (pc[k + 3] - pc[k]);
            } else {
                if (!gze || (kv >= 2 && kv <= g.pnz - 2)) {
                    v = cf.c0z * (pc[k + 2] - pc[k + 1]) + cf.c1z * (pc[k + 3] - pc[k]);
                } else if (kv == 0) {                                     // fwi_2d.c:805 (here r0 == 0)
                    v = g.fs ? (3675.f * pc[3] - 1225.f * pc[4] + 441.f * pc[5] - 75.f * pc[6]) * cf.iz840 : 0.f;
                } else if (kv == 1) {                                     // fwi_2d.c:807
                    v = g.fs ? (-1085.f * pc[3] + 1015.f * pc[4] - 63.f * pc[5] + 5.f * pc[6]) * cf.iz840
                             : cf.iz * (pc[4] - pc[3]);
                } else if (kv == g.pnz - 1) {                             // fwi_2d.c:809
                    v = (pc[k + 2] - pc[k + 1]) * cf.iz;
                } else {
                    v = 0.f;
                }
                const PsiRowSite e = tbz.zv[r0l + k];                       // fwi_2d.c:816-817 (v0: top, all sides)
                if (e.off >= 0 && cin) {
                    const float ps = e.b * pvv[k] + e.a * v;
                    if (k >= 1 && k <= R && kv < g.pnz) *GP(psw + e.off + c) = ps;
                    v += ps;
                }
            }
            vv[k] = v;
        }
        #pragma unroll
        for (int i = 0; i < R; ++i) {
            const int row = r0 + i;
            const int ubase = (r0l + i) * UWP + 1 - x0;                     // + u position = su index
            #define UR(j) su[SIDX(ubase + (j), TZ * UWP)]
            float vz, ux;
            if (!gzw) {
                vz = cf.c0z * (vv[i + 2] - vv[i + 1]) + cf.c1z * (vv[i + 3] - vv[i]);
            } else {
                if (!gze || (row >= 1 && row <= g.pnz - 2)) {
                    vz = cf.c0z * (vv[i + 2] - vv[i + 1]) + cf.c1z * (vv[i + 3] - vv[i]);
                } else if (row == 0) {                                    // fwi_2d.c:848 (i == 0 here)
                    if (i == 0) {
                        vz = g.fs ? (-22.f * vv[1] + 17.f * vv[2] + 9.f * vv[3] - 5.f * vv[4] + vv[5]) * cf.iz24
                                  : (vv[2] - vv[1]) * cf.iz;
                    } else {
                        vz = 0.f;
                    }
                } else if (row == g.pnz - 1) {                            // fwi_2d.c:849
                    vz = (vv[i + 2] - vv[i + 1]) * cf.iz;
                } else {
                    vz = 0.f;
                }
            }
            if (!GX) {
                ux = dxx7(sp, (r0l + i + HZ) * SPW + HX + cl, cf);
            } else if (!gxc) {
                ux = cf.c0x * (UR(c + 1) - UR(c)) + cf.c1x * (UR(c + 2) - UR(c - 1));
            } else {
                if (c >= 1 && c <= g.pnx - 2) {
                    ux = cf.c0x * (UR(c + 1) - UR(c)) + cf.c1x * (UR(c + 2) - UR(c - 1));
                } else if (c == 0) {                                      // fwi_2d.c:829
                    ux = (UR(1) - UR(0)) * cf.ix;
                } else if (c == g.pnx - 1) {                              // fwi_2d.c:831
                    ux = (UR(g.pnx) - UR(g.pnx - 1)) * cf.ix;
                } else {
                    ux = 0.f;
                }
            }
            #undef UR
            const bool inside = (!GZ || row < g.pnz) && (!GX || (c >= 0 && c < g.pnx));
            if (inside && xoff >= 0) {                                    // fwi_2d.c:838-842
                const PsiRowSite e = tbx.xux[cl + 3];
                const float ps = e.b * pux[i] + e.a * ux;
                *GP(psw + xoff + row * np) = ps;
                ux += ps;
            }
            if (gzw && inside) {
                const PsiRowSite e = tbz.zvz[r0l + i + 3];                  // fwi_2d.c:860-861
                if (e.off >= 0) {
                    const float ps = e.b * pvz[i] + e.a * vz;
                    *GP(psw + e.off + c) = ps;
                    vz += ps;
                }
            }
            if (inside) {
                const long long o = (long long)row * g.ld + c;
                float pn = fmaf(kq[i], ux + vz, fmaf(2.f, pc[i + 3], -po[i]));      // fwi_2d.c:878
                if (row == sd.src_r && c == sd.src_c) pn += amp * kq[i];
                *GP(pold + o) = pn;
                if (strip_rows || strip_col) save_strip(P, sd, row, c, pn, P.step);
            }
        }
    }
}

// Forward step, tiles of the general path (edges, CPML, strips) of one
// class (GX, GZ), from the list P.gen_tiles.  MINB (here and on k_fwd_fast,
// k_bwd_edge, k_bwd_int): the resident blocks per SM that the register
// budget is sized for; the engine instantiates the variants its tuning
// (fwi_tuning) chooses from.
template <bool GX, bool GZ, int MINB>
__global__ void __launch_bounds__(NTH, MINB) k_fwd_gen(const StepParams P)
{
    __shared__ __align__(16) float sp[SPH * SPW];
    __shared__ __align__(16) float su[TZ * UWP];
    __shared__ ZSiteTab tbz;
    __shared__ XSiteTab tbx;
    const Geo& g = P.g;
    // work items (tile, shot), item w = shot * gen_n + tile: one per block on a grid
    // of gen_n x 1 x gen_shots blocks, or a loop over them on a smaller grid
    const int nwork = P.gen_n * P.gen_shots, stride = gridDim.x * gridDim.z;
    for (int w = blockIdx.z * gridDim.x + blockIdx.x; w < nwork; w += stride) {
        if (w >= stride) __syncthreads();                  // the previous item's tables and tiles are read no more
        const int gi = w % P.gen_n, s = P.shot_base + w / P.gen_n;
        FWI_TL(P.step, tl_class(GX, GZ, 4), w, 0);
        const ShotDev sd = *GP(P.shots + s);
        const int2 t = P.gen_arith ? gen_tile_at(g, P.fast_tx0, P.fast_tx1, P.fast_tz0, P.fast_tz1, GX, GZ, gi)
                                   : *GP(P.gen_tiles + gi);
        const int x0 = g.xoff + t.x * TX, z0 = g.zoff + t.y * TZ;
        const int2 zr = (GZ && !GX) ? z_tile_rows(g, z0) : make_int2(0, SPH);
        stage_tile(P.pcur + (long long)s * g.fstride, g, x0, z0, sp, zr.x, zr.y);
        // only active shots are launched; the test waits for nothing the copies need
        if (P.step >= sd.nt) { cp_async_wait(); continue; }
        fill_sites<GX, GZ>(P, x0, z0, tbz, tbx);
        cp_async_wait();
        __syncthreads();
        fwd_tile<GX, GZ>(P, sd, s, x0, z0, sp, su, tbz, tbx);
        FWI_TL_END(P.step, tl_class(GX, GZ, 4), w);
    }
}

// Forward step, interior tiles: no edge, CPML or strip cells, so every cell
// takes the same branch-free stencil, its x part as dxx7 of the staged tile.
// The per-cell loads of p^{it-1} and K are issued before the tile copy so
// that their latencies overlap.
template <int MINB>
__global__ void __launch_bounds__(NTH, MINB) k_fwd_fast(const __grid_constant__ StepParams P)
{
    __shared__ __align__(128) float sp[SPH * SPW];
    __shared__ __align__(8) unsigned long long bar;
    const int s = blockIdx.z + P.shot_base;
    const ShotDev sd = *GP(P.shots + s);
    const Geo& g = P.g;
    const Coef& cf = P.c;
    const int x0 = g.xoff + (P.fast_tx0 + blockIdx.x) * TX, z0 = g.zoff + (P.fast_tz0 + blockIdx.y) * TZ;
    const int tx = threadIdx.x, ty = threadIdx.y;
    const long long so = (long long)s * g.fstride;
    const int r0l = R * ty, r0 = z0 + r0l;
    [[maybe_unused]] const long long tl_item = ((long long)blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x;
    FWI_TL(P.step, 4, tl_item, 0);
    // this thread's cells: rows r0 + i, columns x0 + tx + BX h, at 32-bit offsets i ld + BX h
    const long long o0 = (long long)r0 * g.ld + x0 + tx;
    float* __restrict__ prow = P.pold + so + o0;
    const float* __restrict__ krow = P.K + o0;
#ifndef FWI_CPU_EMU
    if (ty == 0 && tx == 0) mbar_init(&bar);
    __syncthreads();
    if (ty == 0 && tx == 0) {                             // the tile of p^it, one TMA copy
        mbar_expect_tx(&bar, TILE_BYTES);
        tma_tile(sp, &P.tm_pcur, g, x0, z0, s, &bar);
    }
#endif
    float po[CX * R], kk[CX * R];
    #pragma unroll
    for (int h = 0; h < CX; ++h)
        #pragma unroll
        for (int i = 0; i < R; ++i) {
            po[h * R + i] = __ldcg(GP(prow + i * g.ld + BX * h));
            kk[h * R + i] = __ldg(GP(krow + i * g.ld + BX * h));
        }
#ifdef FWI_CPU_EMU
    stage_tile(P.pcur + so, g, x0, z0, sp);
    __syncthreads();
    if (P.step >= sd.nt) return;
#else
    // the block leaves only after its copy has landed (or timed out, uniformly);
    // only active shots are launched, so the shot test never fires
    if (__syncthreads_or(!tma_wait(&bar, P.err)) || P.step >= sd.nt) return;
#endif
    const float amp = *GP(P.wav + sd.wav_off + P.step) * cf.iarea;
    const bool src_tile = sd.src_r >= z0 && sd.src_r < z0 + TZ && sd.src_c >= x0 && sd.src_c < x0 + TX;   // uniform
    #pragma unroll
    for (int h = 0; h < CX; ++h) {
        const int cl = tx + BX * h, c = x0 + cl;
        float pc[R + 6];
        #pragma unroll
        for (int k = 0; k < R + 6; ++k) pc[k] = sp[SIDX((r0l + k) * SPW + HX + cl, SPH * SPW)];
        float vv[R + 3];
        #pragma unroll
        for (int k = 0; k < R + 3; ++k) vv[k] = cf.c0z * (pc[k + 2] - pc[k + 1]) + cf.c1z * (pc[k + 3] - pc[k]);
        #pragma unroll
        for (int i = 0; i < R; ++i) {
            const int row = r0 + i;
            const float vz = cf.c0z * (vv[i + 2] - vv[i + 1]) + cf.c1z * (vv[i + 3] - vv[i]);
            const float ux = dxx7(sp, (r0l + i + HZ) * SPW + HX + cl, cf);
            const float k1 = kk[h * R + i];
            float pn = fmaf(k1, ux + vz, fmaf(2.f, pc[i + 3], -po[h * R + i]));
            if (src_tile && row == sd.src_r && c == sd.src_c) pn += amp * k1;
            __stcg(GP(prow + i * g.ld + BX * h), pn);
        }
    }
    FWI_TL_END(P.step, 4, tl_item);
}

// syn[r][it/jump] = p^{it+1}(receiver r) for every receiver of the launched shots.
__global__ void k_sample(const RecParams Q)
{
    const int i = Q.lo + blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= Q.hi) return;
    const RecSample r = *GP(Q.recs + i);
    if (Q.step >= GP(Q.shots + r.slot)->nt) return;
    *GP(Q.syn + r.syn_base + Q.step / Q.jump) = *GP(Q.field + (long long)r.slot * Q.g.fstride + r.foff);
}

// ---------------------------------------------------------------------------
// Backward step: adjoint + rebuild + imaging
// ---------------------------------------------------------------------------
// srx is the last member: tiles without x-general work are launched with
// offsetof(BwdSmem, srx) dynamic bytes and never touch it.
struct BwdSmem {
    float sq[SPH * SPW];   // b^{m+1} tile + halo
    float sp[SPH * SPW];   // p^{m-1} tile + halo
    float racc[TZ * TX];   // receiver adjoint sources of the tile
    ZSiteTab tbz;          // z psi sites of the tile
    // x-general tiles and corners only: z-only tiles are launched without these
    float su[TZ * UWP];    // adjoint ubar, then rebuild u
    float srx[TZ * RXP];   // adjoint x-stage input (psi-adjusted b)
    XSiteTab tbx;          // x psi sites of the tile
};

// All shared-memory accesses below use integer indices relative to the start
// of their array (global column jg of the tile row sits at jg - x0 + offset),
// so no pointer is ever formed outside the array it points into.
//
// One adjoint tile; GX / GZ select the general formulas along x / z as in
// fwd_tile.  Rows past pnz and column halves past pnx are skipped (uniform
// per warp); `live` tells the caller whether this thread's rows exist.
template <bool GX, bool GZ>
__device__ __forceinline__ void adj_tile(const StepParams& P, const ShotDev& sd, int s, int x0, int z0,
                                         BwdSmem& sm, bool do_res, float* bm)
{
    const Geo& g = P.g;
    const Coef& cf = P.c;
    const ZSiteTab& tbz = sm.tbz;
    const XSiteTab& tbx = sm.tbx;
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int np = g.npml, pnx = g.pnx, pnz = g.pnz;
    const long long so = (long long)s * g.fstride;
    const float* __restrict__ psr = P.psr + (long long)s * P.pl.stride;
    float* __restrict__ psw = P.psw + (long long)s * P.pl.stride;
    [[maybe_unused]] constexpr int NS = SPH * SPW, NU = TZ * UWP, NR = TZ * RXP;

    // psi entries of both x stages first (independent loads): the ux
    // recursion at cells i = x0-3+ii and the u recursion at positions
    // j = x0-1+jj of the x-general column halves
    float pux[R][3], pu[R][3];
    if (GX) {
        #pragma unroll
        for (int k = 0; k < R; ++k) {
            const int row = z0 + ty + BY * k;
            const bool live = !(GZ && (row < 0 || row >= pnz));
            #pragma unroll
            for (int h = 0; h < 3; ++h) {
                const int ii = tx + BX * h, jj = ii;
                const int xo = (live && ii < RXW && !x_window_outside(x0 - 3 + BX * h, BX, 0, pnx - 1))
                                   ? tbx.xux[ii].off : -1;
                pux[k][h] = xo >= 0 ? __ldcg(GP(psr + xo + row * np)) : 0.f;
                const bool gen = live && jj < UW && x_window_general(g, x0 - 1 + BX * h, BX) &&
                                 !x_window_outside(x0 - 1 + BX * h, BX, 0, pnx);
                const int uo = gen ? tbx.xu[jj].off : -1;
                pu[k][h] = uo >= 0 ? __ldcg(GP(psr + uo + row * (np + 1))) : 0.f;
            }
        }
    }

    // x stage 1 (x-general tiles): rbar = q adjusted by the adjoint of the ux psi recursion
    if (GX) {
        #pragma unroll
        for (int k = 0; k < R; ++k) {
            const int rl = ty + BY * k, row = z0 + rl;
            if (GZ && (row < 0 || row >= pnz)) continue;
            const int qrow = (rl + HZ) * SPW + HX - 3;        // sq index of column x0 - 3
            #pragma unroll
            for (int h = 0; h < 3; ++h) {
                const int ii = tx + BX * h;
                if (ii >= RXW) break;
                if (x_window_outside(x0 - 3 + BX * h, BX, 0, pnx - 1)) continue;   // stage 2 reads cells 0 .. pnx-1
                float r = sm.sq[SIDX(qrow + ii, NS)];
                const PsiRowSite e = tbx.xux[ii];
                if (e.off >= 0) {
                    const float tt = r + pux[k][h];
                    r = r + e.a * tt;
                    if (ii >= 3 && ii < 3 + TX) *GP(psw + e.off + row * np) = e.b * tt;
                }
                sm.srx[SIDX(rl * RXP + ii, NR)] = r;
            }
        }
        __syncthreads();
    }
    // x stage 2: ubar at u positions j in [x0-1, x0+TX+1], x-general tiles only
    // (elsewhere the adjoint x part is dxx7 of sq)
    #pragma unroll
    for (int k = 0; k < R; ++k) {
        if (!GX) break;
        const int rl = ty + BY * k, row = z0 + rl;
        if (GZ && (row < 0 || row >= pnz)) continue;
        #pragma unroll
        for (int h = 0; h < 3; ++h) {
            const int jj = tx + BX * h;
            if (jj >= UW) break;
            const int j = x0 - 1 + jj;
            float ub;
            if (!GX || !x_window_general(g, x0 - 1 + BX * h, BX)) {        // plain ubar for this column half
                const int q0 = (rl + HZ) * SPW + HX - 1 + jj;     // sq index of column j
                ub = cf.c0x * (sm.sq[SIDX(q0 - 1, NS)] - sm.sq[SIDX(q0, NS)]) +
                     cf.c1x * (sm.sq[SIDX(q0 - 2, NS)] - sm.sq[SIDX(q0 + 1, NS)]);
            } else if (x_window_outside(x0 - 1 + BX * h, BX, 0, pnx)) {    // ubar positions are 0 .. pnx
                ub = 0.f;
            } else {
                const int rbase = rl * RXP + 3 - x0;             // + global column = srx index
                #define RM(i) (((i) >= 1 && (i) <= pnx - 2) ? sm.srx[SIDX(rbase + (i), NR)] : 0.f)
                ub = cf.c0x * (RM(j - 1) - RM(j)) + cf.c1x * (RM(j - 2) - RM(j + 1));
                #undef RM
                if (j == 1) ub += cf.ix * sm.srx[SIDX(rbase, NR)];
                if (j == 0) ub -= cf.ix * sm.srx[SIDX(rbase, NR)];
                if (j == pnx) ub += cf.ix * sm.srx[SIDX(rbase + pnx - 1, NR)];
                if (j == pnx - 1) ub -= cf.ix * sm.srx[SIDX(rbase + pnx - 1, NR)];
                const PsiRowSite e = tbx.xu[jj];
                if (e.off >= 0) {
                    const float tt = ub + pu[k][h];
                    ub = ub + e.a * tt;
                    if (jj >= 1 && jj <= TX) *GP(psw + e.off + row * (np + 1)) = e.b * tt;
                }
            }
            sm.su[SIDX(rl * UWP + jj, NU)] = ub;
        }
    }
    if (GX) __syncthreads();

    const float* __restrict__ K = P.K;
    float* __restrict__ bold = P.bold + so;
    #pragma unroll
    for (int q = 0; q < CX; ++q) {
        const ZUnit zu = z_unit<GZ>(g, z0, q);                              // the rebuild takes the same units
        if (!zu.live) continue;
        const int r0l = zu.r0l, r0 = z0 + r0l, h = zu.h;
        const bool gzw = GZ && z_window_general(g, r0, R);                 // this unit's rows need the z-general formulas
        const bool gze = gzw && z_unit_edge(g, r0);                        // ... and the grid-edge ones among them
        if (GX && (x0 + BX * h >= pnx || x0 + BX * h + BX <= 0)) continue;   // column half outside the grid
        const bool gxc = GX && x_window_general(g, x0 + BX * h, BX);        // this half needs the x-general formulas
        const int cl = tx + BX * h, c = x0 + cl;
        const bool zs = gzw && (!GX || (c >= 0 && c < pnx));               // z sites exist in grid columns only
        // every global operand of this column segment first: K, b^{m+2} and the psi entries
        float kq[R], bo[R], prz[R + 6], pvb[R + 3];
        #pragma unroll
        for (int i = 0; i < R; ++i) {
            const int row = r0 + i;
            const bool inside = (!GZ || row < pnz) && (!GX || (c >= 0 && c < pnx));
            const long long o = (long long)row * g.ld + c;
            kq[i] = inside ? __ldg(GP(K + o)) : 0.f;
            bo[i] = inside ? *GP(bold + o) : 0.f;
        }
        #pragma unroll
        for (int k = 0; k < R + 6; ++k) {
            const int off = zs ? tbz.zvz[r0l + k].off : -1;
            prz[k] = off >= 0 ? __ldcg(GP(psr + off + c)) : 0.f;
        }
        #pragma unroll
        for (int k = 0; k < R + 3; ++k) {
            const int off = zs ? tbz.zv[r0l + k].off : -1;
            pvb[k] = off >= 0 ? __ldcg(GP(psr + off + c)) : 0.f;
        }

        float qc[R + 6];
        #pragma unroll
        for (int k = 0; k < R + 6; ++k) qc[k] = sm.sq[SIDX((r0l + k) * SPW + HX + cl, NS)];   // rows r0-3+k
        float rz[R + 6];
        #pragma unroll
        for (int k = 0; k < R + 6; ++k) {
            float r = qc[k];
            if (zs) {
                const PsiRowSite e = tbz.zvz[r0l + k];
                if (e.off >= 0) {
                    const float tt = r + prz[k];
                    r = r + e.a * tt;
                    if (k >= 3 && k < 3 + R) *GP(psw + e.off + c) = e.b * tt;
                }
            }
            rz[k] = r;
        }
        float vb[R + 3];                                                  // vbar rows r0-1+k
        #pragma unroll
        for (int k = 0; k < R + 3; ++k) {
            const int kv = r0 - 1 + k;
            float v;
            if (!gze) {
                v = cf.c0z * (rz[k + 1] - rz[k + 2]) + cf.c1z * (rz[k] - rz[k + 3]);
            } else {
                // rz index of row q is q - (r0 - 3); row kv-1 -> k+1 etc.
                const float m1 = (kv - 1 >= 1 && kv - 1 <= pnz - 2) ? rz[k + 1] : 0.f;
                const float m0 = (kv     >= 1 && kv     <= pnz - 2) ? rz[k + 2] : 0.f;
                const float m2 = (kv - 2 >= 1 && kv - 2 <= pnz - 2) ? rz[k]     : 0.f;
                const float p1 = (kv + 1 >= 1 && kv + 1 <= pnz - 2) ? rz[k + 3] : 0.f;
                v = cf.c0z * (m1 - m0) + cf.c1z * (m2 - p1);
                if (g.fs) {
                    if (kv >= 0 && kv <= 4) {
                        // vz[0] = (-22 v0 + 17 v1 + 9 v2 - 5 v3 + v4) iz24 (fwi_2d.c:848), transposed;
                        // kv <= 4 only happens in the top tile (z0 <= 0), where row 0 is sq row HZ - z0
                        const float r00 = sm.sq[SIDX((HZ - z0) * SPW + HX + cl, NS)];   // rbar[0] = q[0] (no top CPML)
                        const float hcoef = (kv == 0) ? -22.f : (kv == 1) ? 17.f : (kv == 2) ? 9.f : (kv == 3) ? -5.f : 1.f;
                        v += hcoef * r00 * cf.iz24;
                    }
                } else {
                    if (kv == 1) v += cf.iz * rz[3];      // r0 == 0 here: row 0 sits at index 3
                    if (kv == 0) v -= cf.iz * rz[3];
                }
                if (kv == pnz) v += cf.iz * rz[k + 1];
                if (kv == pnz - 1) v -= cf.iz * rz[k + 2];
            }
            if (zs) {
                const PsiRowSite e = tbz.zv[r0l + k];
                if (e.off >= 0) {
                    const float tt = v + pvb[k];
                    v = v + e.a * tt;
                    if (k >= 1 && k <= R && kv < pnz) *GP(psw + e.off + c) = e.b * tt;
                }
            }
            vb[k] = v;
        }
        #pragma unroll
        for (int i = 0; i < R; ++i) {
            const int row = r0 + i;
            const int ubase = (r0l + i) * UWP + 1 - x0;                   // + u position = su index
            #define UB(j) sm.su[SIDX(ubase + (j), NU)]
            float pz, px;
            if (!gze) {
                pz = cf.c0z * (vb[i + 1] - vb[i + 2]) + cf.c1z * (vb[i] - vb[i + 3]);
            } else {
                // vbar index of row q is q - (r0 - 1)
                const float M0 = (row     >= 2 && row     <= pnz - 2) ? vb[i + 1] : 0.f;
                const float M1 = (row + 1 >= 2 && row + 1 <= pnz - 2) ? vb[i + 2] : 0.f;
                const float Mm = (row - 1 >= 2 && row - 1 <= pnz - 2) ? vb[i]     : 0.f;
                const float M2 = (row + 2 >= 2 && row + 2 <= pnz - 2) ? vb[i + 3] : 0.f;
                pz = cf.c0z * (M0 - M1) + cf.c1z * (Mm - M2);
                if (row >= 0 && row <= 3 && i == row) {                     // r0 == 0: vbar[0], vbar[1] at 1, 2
                    if (g.fs) {
                        const float g0 = (row == 0) ? 3675.f : (row == 1) ? -1225.f : (row == 2) ? 441.f : -75.f;
                        const float g1 = (row == 0) ? -1085.f : (row == 1) ? 1015.f : (row == 2) ? -63.f : 5.f;
                        pz += (g0 * vb[1] + g1 * vb[2]) * cf.iz840;
                    } else {
                        if (row == 1) pz += cf.iz * vb[2];
                        if (row == 0) pz -= cf.iz * vb[2];
                    }
                }
                if (row == pnz - 1) pz += cf.iz * vb[i + 1];
                if (row == pnz - 2) pz -= cf.iz * vb[i + 2];
            }
            if (!GX) {
                px = dxx7(sm.sq, (r0l + i + HZ) * SPW + HX + cl, cf);
            } else if (!gxc) {
                px = cf.c0x * (UB(c) - UB(c + 1)) + cf.c1x * (UB(c - 1) - UB(c + 2));
            } else {
                #define UM(j) (((j) >= 2 && (j) <= pnx - 2) ? UB(j) : 0.f)
                px = cf.c0x * (UM(c) - UM(c + 1)) + cf.c1x * (UM(c - 1) - UM(c + 2));
                #undef UM
                if (c == 1) px += cf.ix * UB(1);
                if (c == 0) px -= cf.ix * UB(1);
                if (c == pnx - 1) px += cf.ix * UB(pnx - 1);
                if (c == pnx - 2) px -= cf.ix * UB(pnx - 1);
            }
            #undef UB
            float pbar = px + pz;
            if (do_res) pbar += sm.racc[SIDX((r0l + i) * TX + cl, TZ * TX)];
            float b = 0.f;
            if ((!GZ || row < pnz) && (!GX || (c >= 0 && c < pnx))) {
                const long long o = (long long)row * g.ld + c;
                b = fmaf(kq[i], pbar, fmaf(2.f, qc[i + 3], -bo[i]));
                *GP(bold + o) = b;
            }
            bm[q * R + i] = b;
        }
    }
}

// One general backward tile (edges, CPML, strips): general tile gi of the
// class (GX, GZ), shot slot s.
template <bool GX, bool GZ>
__device__ __forceinline__ void bwd_edge_item(const StepParams& P, BwdSmem& sm, int gi, int s)
{
    const Geo& g = P.g;
    const int2 t = P.gen_arith ? gen_tile_at(g, P.fast_tx0, P.fast_tx1, P.fast_tz0, P.fast_tz1, GX, GZ, gi)
                               : *GP(P.gen_tiles + gi);
    const int x0 = g.xoff + t.x * TX, z0 = g.zoff + t.y * TZ;
    const ShotDev sd = *GP(P.shots + s);
    const int m = P.step;
    const Coef& cf = P.c;
    const int tile = t.y * g.ntx + t.x;
    const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * BX + tx;
    const long long so = (long long)s * g.fstride;
    [[maybe_unused]] constexpr int NS = SPH * SPW, NU = TZ * UWP;

    // physical region and the rebuilt interior (3 cells inside it)
    const int zp0 = g.z0p, zp1 = g.z0p + g.nz, xp0 = g.x0p, xp1 = g.x0p + g.nx;
    const bool phys = z0 < zp1 && z0 + TZ > zp0 && x0 < xp1 && x0 + TX > xp0;

    const int2 zr = (GZ && !GX) ? z_tile_rows(g, z0) : make_int2(0, SPH);
    stage_tile(P.bcur + so, g, x0, z0, sm.sq, zr.x, zr.y);
    if (phys) stage_tile(P.pcur + so, g, x0, z0, sm.sp, zr.x, zr.y);
    // only active shots are launched; the test comes after the copies are issued
    if (m > sd.nt) { cp_async_wait(); return; }

    // adjoint sources r^m at the receivers when m-1 = k*jump
    const int rb = *GP(P.rtile + sd.rtile_off + tile), re = *GP(P.rtile + sd.rtile_off + tile + 1);
    const bool do_res = re > rb && ((m - 1) % P.jump) == 0;
    if (do_res) {
        for (int q = tid; q < TZ * TX; q += NTH) sm.racc[SIDX(q, TZ * TX)] = 0.f;
        __syncthreads();
        gather_residuals(P, rb, re, (m - 1) / P.jump, sm.racc);
    }
    fill_sites<GX, GZ>(P, x0, z0, sm.tbz, sm.tbx);
    cp_async_wait();
    __syncthreads();

    float bm[CX * R];
    adj_tile<GX, GZ>(P, sd, s, x0, z0, sm, do_res, bm);
    if (!phys) return;   // uniform per block

    // rebuild of p^{m-2} and imaging (physical cells only); the u positions
    // of p^{m-1} into su for x-general tiles (elsewhere the x part is dxx7 of sp)
    if (GX) __syncthreads();     // su is reused
    #pragma unroll
    for (int k = 0; k < R; ++k) {
        if (!GX) break;
        const int rl = ty + BY * k;
        if (GZ && (z0 + rl < zp0 || z0 + rl >= zp1)) continue;
        #pragma unroll
        for (int h = 0; h < 3; ++h) {
            const int jj = tx + BX * h;
            if (jj >= UW) break;
            const int p0 = (rl + HZ) * SPW + HX - 1 + jj;      // sp index of column j = x0 - 1 + jj
            sm.su[SIDX(rl * UWP + jj, NU)] = cf.c0x * (sm.sp[SIDX(p0, NS)] - sm.sp[SIDX(p0 - 1, NS)]) +
                                             cf.c1x * (sm.sp[SIDX(p0 + 1, NS)] - sm.sp[SIDX(p0 - 2, NS)]);
        }
    }
    if (GX) __syncthreads();
    const float* __restrict__ K = P.K;
    float* __restrict__ pold = P.pold + so;
    float* __restrict__ gacc = P.gacc + so;
    const float f = *GP(P.wav + sd.wav_off + m - 1) * cf.iarea;
    #pragma unroll
    for (int q = 0; q < CX; ++q) {
        const ZUnit zu = z_unit<GZ>(g, z0, q);               // adj_tile's units: bm[q] belongs to this one
        const int r0l = zu.r0l, r0 = z0 + r0l, h = zu.h;
        if (!zu.live || (GZ && (r0 >= zp1 || r0 + R <= zp0))) continue;   // no physical row; no barrier follows
        const bool gzw = GZ && z_window_general(g, r0, R);  // rows that may be outside the region or strips
        if (GX && (x0 + BX * h >= xp1 || x0 + BX * h + BX <= xp0)) continue;   // no physical column in this half
        const bool gxc = GX && x_window_general(g, x0 + BX * h, BX);
        const int cl = tx + BX * h, c = x0 + cl;
        const int ix = c - g.x0p;
        if (gxc && (ix < 0 || ix >= g.nx)) continue;
        // every global operand of this column segment first: K, p^m, g and the strip values
        float kq[R], pmq[R], gq[R], pst[R];
        #pragma unroll
        for (int i = 0; i < R; ++i) {
            const int row = r0 + i, iz = row - g.z0p;
            const bool live = !(gzw && (iz < 0 || iz >= g.nz));
            const bool strip = (gzw && (iz < NSTRIP || iz >= g.nz - NSTRIP)) || (gxc && (ix < NSTRIP || ix >= g.nx - NSTRIP));
            const long long o = (long long)row * g.ld + c;
            kq[i] = live ? __ldg(GP(K + o)) : 1.f;
            pmq[i] = live ? *GP(pold + o) : 0.f;
            gq[i] = live ? *GP(gacc + o) : 0.f;
            pst[i] = (live && strip && m - 3 >= 0) ? load_strip(P, sd, iz, ix, m - 3) : 0.f;
        }
        float pc[R + 6];
        #pragma unroll
        for (int k = 0; k < R + 6; ++k) pc[k] = sm.sp[SIDX((r0l + k) * SPW + HX + cl, NS)];
        float vv[R + 3];
        #pragma unroll
        for (int k = 0; k < R + 3; ++k) vv[k] = cf.c0z * (pc[k + 2] - pc[k + 1]) + cf.c1z * (pc[k + 3] - pc[k]);
        #pragma unroll
        for (int i = 0; i < R; ++i) {
            const int row = r0 + i, iz = row - g.z0p;
            if (gzw && (iz < 0 || iz >= g.nz)) continue;
            const long long o = (long long)row * g.ld + c;
            const float kk = kq[i];
            const float pm = pmq[i];             // p^m
            const float p1 = pc[i + 3];          // p^{m-1}
            float pn, lp;
            const bool strip = (gzw && (iz < NSTRIP || iz >= g.nz - NSTRIP)) || (gxc && (ix < NSTRIP || ix >= g.nx - NSTRIP));
            if (!strip) {
                const int u0 = (r0l + i) * UWP + 1 + cl;        // su index of u position c
                const float vz = cf.c0z * (vv[i + 2] - vv[i + 1]) + cf.c1z * (vv[i + 3] - vv[i]);
                const float ux = GX ? cf.c0x * (sm.su[SIDX(u0 + 1, NU)] - sm.su[SIDX(u0, NU)]) +
                                          cf.c1x * (sm.su[SIDX(u0 + 2, NU)] - sm.su[SIDX(u0 - 1, NU)])
                                    : dxx7(sm.sp, (r0l + i + HZ) * SPW + HX + cl, cf);
                const float w = ux + vz;
                pn = fmaf(kk, w, fmaf(2.f, p1, -pm));
                lp = w;
                if (row == sd.src_r && c == sd.src_c) { pn += f * kk; lp += f; }
            } else {
                pn = pst[i];
                lp = ((pm - 2.f * p1) + pn) / kk;
            }
            *GP(pold + o) = pn;
            *GP(gacc + o) = fmaf(bm[q * R + i], lp, gq[i]);
        }
    }
}

// Backward step, the tiles of one general class (GX, GZ) from the list
// P.gen_tiles (or gen_tile_at), for the launch's shots.
template <bool GX, bool GZ, int MINB>
__global__ void __launch_bounds__(NTH, MINB) k_bwd_edge(const StepParams P)
{
    FWI_DYN_SMEM(smraw);
    BwdSmem& sm = *reinterpret_cast<BwdSmem*>(smraw);
    // work items (tile, shot) as in k_fwd_gen
    const int nwork = P.gen_n * P.gen_shots, stride = gridDim.x * gridDim.z;
    for (int w = blockIdx.z * gridDim.x + blockIdx.x; w < nwork; w += stride) {
        if (w >= stride) __syncthreads();                  // the previous item's shared memory is read no more
        FWI_TL(P.step, tl_class(GX, GZ, 0), w, 0);
        bwd_edge_item<GX, GZ>(P, sm, w % P.gen_n, P.shot_base + w / P.gen_n);
        FWI_TL_END(P.step, tl_class(GX, GZ, 0), w);
    }
}

// Shared memory of an interior backward tile: the x parts are dxx7 of the
// staged tiles, so interior blocks need neither u positions nor a
// psi-adjusted copy (sizeof(BwdIntSmem) dynamic bytes).
constexpr int SPA = (SPH * SPW + 31) / 32 * 32;   // staged tile padded to 128 bytes
struct BwdIntSmem {
    float sq[SPA];         // b^{m+1} tile + halo (TMA destination, 128-byte aligned)
    float sp[SPA];         // p^{m-1} tile + halo
    float racc[TZ * TX];   // receiver adjoint sources of the tile
    unsigned long long bar;   // mbarrier of the two tile copies
};
// Launch size of k_bwd_int: the layout plus room to align it to 128 bytes.
constexpr size_t BWD_INT_SMEM = sizeof(BwdIntSmem) + 128;

// Backward step, interior tiles (the rectangle fast_tx0.. x fast_tz0..):
// every cell and stencil neighbour is a physical interior cell (no CPML,
// edge formula or strip), so the adjoint is L^T b = the staggered
// differences with their signs exchanged, the rebuild is the interior
// operator, and the imaging term is the rebuild's own stencil value.  The
// x parts are dxx7 of the staged tiles, so one barrier (after the tile
// copies) is all the block needs.  b^{m+2} and K are loaded into registers
// at block start, with the tile copies; p^m and g of a column half as soon
// as the half's adjoint values are out (1.6% faster than at block start,
// where they spill).
// (Copying p^m and g into shared memory instead was 5% slower: 55 KB per
// block leaves too little of the SM's shared memory and L1 for the
// concurrent general blocks.)
template <int MINB>
__global__ void __launch_bounds__(NTH, MINB) k_bwd_int(const __grid_constant__ StepParams P)
{
    FWI_DYN_SMEM(smraw);
#ifdef FWI_CPU_EMU
    BwdIntSmem& sm = *reinterpret_cast<BwdIntSmem*>(smraw);
#else
    BwdIntSmem& sm = *reinterpret_cast<BwdIntSmem*>(smraw + ((128u - (smem_u32(smraw) & 127u)) & 127u));
#endif
    const Geo& g = P.g;
    const Coef& cf = P.c;
    const int s = blockIdx.z + P.shot_base;
    const ShotDev sd = *GP(P.shots + s);
    const int m = P.step;
    const int txi = P.fast_tx0 + blockIdx.x, tzi = P.fast_tz0 + blockIdx.y;
    const int x0 = g.xoff + txi * TX, z0 = g.zoff + tzi * TZ;
    const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * BX + tx;
    const long long so = (long long)s * g.fstride;
    float* __restrict__ bold = P.bold + so;
    float* __restrict__ pold = P.pold + so;
    float* __restrict__ gacc = P.gacc + so;
    const int r0l = R * ty, r0 = z0 + r0l;
    [[maybe_unused]] constexpr int NS = SPH * SPW;
    [[maybe_unused]] const long long tl_item = ((long long)blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x;
    FWI_TL(P.step, 0, tl_item, 0);

#ifndef FWI_CPU_EMU
    if (tid == 0) mbar_init(&sm.bar);
    __syncthreads();
    if (tid == 0) {                                       // the tiles of b^{m+1} and p^{m-1}, two TMA copies
        mbar_expect_tx(&sm.bar, 2 * TILE_BYTES);
        tma_tile(sm.sq, &P.tm_bcur, g, x0, z0, s, &sm.bar);
        tma_tile(sm.sp, &P.tm_pcur, g, x0, z0, s, &sm.bar);
    }
#endif
    float bo[CX * R], kk[CX * R], pm[CX * R], ga[CX * R];
    #pragma unroll
    for (int h = 0; h < CX; ++h)
        #pragma unroll
        for (int i = 0; i < R; ++i) {
            const long long o = (long long)(r0 + i) * g.ld + x0 + tx + BX * h;
            bo[h * R + i] = __ldcg(GP(bold + o));
            kk[h * R + i] = __ldg(GP(P.K + o));
        }
#ifdef FWI_CPU_EMU
    stage_tile(P.bcur + so, g, x0, z0, sm.sq);
    stage_tile(P.pcur + so, g, x0, z0, sm.sp);
    if (m > sd.nt) return;
#else
    // only active shots are launched; the test comes after the loads are issued
    // (a block leaves only after its copies have landed)
    if (m > sd.nt) { __syncthreads_or(!tma_wait(&sm.bar, P.err)); return; }
#endif

    // adjoint sources r^m at the receivers when m-1 = k*jump
    const int tile = tzi * g.ntx + txi;
    const int rb = *GP(P.rtile + sd.rtile_off + tile), re = *GP(P.rtile + sd.rtile_off + tile + 1);
    const bool do_res = re > rb && ((m - 1) % P.jump) == 0;
    if (do_res) {
        for (int q = tid; q < TZ * TX; q += NTH) sm.racc[SIDX(q, TZ * TX)] = 0.f;
        __syncthreads();
        gather_residuals(P, rb, re, (m - 1) / P.jump, sm.racc);
    }
#ifdef FWI_CPU_EMU
    __syncthreads();
#else
    if (__syncthreads_or(!tma_wait(&sm.bar, P.err))) return;   // uniform: every thread saw the same barrier
#endif

    // adjoint: the z chain in registers, the x part as dxx7 of b^{m+1} (the
    // interior operator is symmetric), and b^m = 2 b^{m+1} - b^{m+2} + K (L^T b^{m+1} + r^m)
    float bm[CX * R];
    #pragma unroll
    for (int h = 0; h < CX; ++h) {
        const int cl = tx + BX * h, c = x0 + cl;
        float qc[R + 6];
        #pragma unroll
        for (int k = 0; k < R + 6; ++k) qc[k] = sm.sq[SIDX((r0l + k) * SPW + HX + cl, NS)];   // rows r0-3+k
        float vb[R + 3];
        #pragma unroll
        for (int k = 0; k < R + 3; ++k) vb[k] = cf.c0z * (qc[k + 1] - qc[k + 2]) + cf.c1z * (qc[k] - qc[k + 3]);
        #pragma unroll
        for (int i = 0; i < R; ++i) {
            const float pz = cf.c0z * (vb[i + 1] - vb[i + 2]) + cf.c1z * (vb[i] - vb[i + 3]);
            const float px = dxx7(sm.sq, (r0l + i + HZ) * SPW + HX + cl, cf);
            float pbar = px + pz;
            if (do_res) pbar += sm.racc[SIDX((r0l + i) * TX + cl, TZ * TX)];
            const int q = h * R + i;
            bm[q] = fmaf(kk[q], pbar, fmaf(2.f, qc[i + 3], -bo[q]));
            __stcg(GP(bold + (long long)(r0 + i) * g.ld + c), bm[q]);
        }
        // this half's rebuild operands, in the registers its b^{m+2} leaves free
        #pragma unroll
        for (int i = 0; i < R; ++i) {
            const long long o = (long long)(r0 + i) * g.ld + c;
            pm[h * R + i] = __ldcg(GP(pold + o));
            ga[h * R + i] = __ldcg(GP(gacc + o));
        }
    }

    // rebuild p^{m-2} = 2 p^{m-1} - p^m + K (L p^{m-1} + s^{m-1}) and imaging g += b^m (L p^{m-1} + f^{m-1})
    const float f = *GP(P.wav + sd.wav_off + m - 1) * cf.iarea;
    const bool src_tile = sd.src_r >= z0 && sd.src_r < z0 + TZ && sd.src_c >= x0 && sd.src_c < x0 + TX;   // uniform
    #pragma unroll
    for (int h = 0; h < CX; ++h) {
        const int cl = tx + BX * h, c = x0 + cl;
        float pc[R + 6];
        #pragma unroll
        for (int k = 0; k < R + 6; ++k) pc[k] = sm.sp[SIDX((r0l + k) * SPW + HX + cl, NS)];
        float vv[R + 3];
        #pragma unroll
        for (int k = 0; k < R + 3; ++k) vv[k] = cf.c0z * (pc[k + 2] - pc[k + 1]) + cf.c1z * (pc[k + 3] - pc[k]);
        #pragma unroll
        for (int i = 0; i < R; ++i) {
            const int row = r0 + i, q = h * R + i;
            const long long o = (long long)row * g.ld + c;
            const float vz = cf.c0z * (vv[i + 2] - vv[i + 1]) + cf.c1z * (vv[i + 3] - vv[i]);
            const float ux = dxx7(sm.sp, (r0l + i + HZ) * SPW + HX + cl, cf);
            float lp = ux + vz;
            float pn = fmaf(kk[q], lp, fmaf(2.f, pc[i + 3], -pm[q]));
            if (src_tile && row == sd.src_r && c == sd.src_c) { pn += f * kk[q]; lp += f; }
            __stcg(GP(pold + o), pn);
            __stcg(GP(gacc + o), fmaf(bm[q], lp, ga[q]));
        }
    }
    FWI_TL_END(P.step, 0, tl_item);
}

// ---------------------------------------------------------------------------
// Misfit, model and reduction kernels
// ---------------------------------------------------------------------------

// K = vext^2 dt^2 with vext the edge-replicated model (model_ext /
// model_ext_fs_no, fwi_2d.c:29-107, are clamp extensions).
__global__ void k_build_K(const float* __restrict__ vel, float* __restrict__ K, Geo g, float dt)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    const int r = blockIdx.y;
    if (c >= g.pnx || r >= g.pnz) return;
    const int iz = min(max(r - g.z0p, 0), g.nz - 1);
    const int ix = min(max(c - g.x0p, 0), g.nx - 1);
    const float v = vel[(long long)iz * g.nx + ix];
    K[(long long)r * g.ld + c] = __fmul_rn(__fmul_rn(__fmul_rn(v, v), dt), dt);
}

__device__ __forceinline__ double warp_sum(double v)
{
    #pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// res = syn - obs and per-block partial sums of res^2 (FP64).
__global__ void k_misfit(const float* __restrict__ syn, const float* __restrict__ obs, float* __restrict__ res,
                         long long n, double* __restrict__ partial)
{
    __shared__ double ws[32];
    double acc = 0.0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float r = syn[i] - obs[i];
        res[i] = r;
        acc += (double)r * (double)r;
    }
    acc = warp_sum(acc);
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x < 32) {
        double v = threadIdx.x < (blockDim.x >> 5) ? ws[threadIdx.x] : 0.0;
        v = warp_sum(v);
        if (threadIdx.x == 0) partial[blockIdx.x] = v;
    }
}

// Per-trace variant of k_misfit: block t forms res = syn - obs for trace t
// and writes sum(res^2) of that trace (FP64) to partial[t].
__global__ void k_misfit_traces(const float* __restrict__ syn, const float* __restrict__ obs, float* __restrict__ res,
                                int nsamples, double* __restrict__ partial)
{
    __shared__ double ws[32];
    const long long base = (long long)blockIdx.x * nsamples;
    double acc = 0.0;
    for (int i = threadIdx.x; i < nsamples; i += blockDim.x) {
        const float r = syn[base + i] - obs[base + i];
        res[base + i] = r;
        acc += (double)r * (double)r;
    }
    acc = warp_sum(acc);
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x < 32) {
        double v = threadIdx.x < (blockDim.x >> 5) ? ws[threadIdx.x] : 0.0;
        v = warp_sum(v);
        if (threadIdx.x == 0) partial[blockIdx.x] = v;
    }
}

// out[0] = out[1] = 1/2 sum partial (deterministic single-block sum).
__global__ void k_misfit_final(const double* __restrict__ partial, int n, double* __restrict__ out)
{
    __shared__ double ws[32];
    double acc = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) acc += partial[i];
    acc = warp_sum(acc);
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x < 32) {
        double v = threadIdx.x < (blockDim.x >> 5) ? ws[threadIdx.x] : 0.0;
        v = warp_sum(v);
        if (threadIdx.x == 0) { out[0] = 0.5 * v; out[1] = 0.5 * v; }
    }
}

// ---------------------------------------------------------------------------
// Checkpoints of the forward state (FWI_STORE_SNAPSHOTS)
// ---------------------------------------------------------------------------
// The strips (NS = 2M-1 wide) of field f (p^{t+1}, origin-based field
// layout) into ring slot t - ring_t0, in save_strip's layout: [NS top rows |
// NS bottom rows] x nx, then [NS left columns | NS right columns] x nz, for
// shots shot_base + blockIdx.z.  Used after a checkpoint is restored, for the two time levels
// it holds.
template <int NS>
__global__ void k_strips_of_field(const StepParams P, const float* __restrict__ f, int t)
{
    const Geo& g = P.g;
    const int s = blockIdx.z + P.shot_base;
    const ShotDev sd = *GP(P.shots + s);
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    const int nud = 2 * NS * g.nx;
    if (e >= P.strip_len) return;
    int iz, ix;
    if (e < nud) {
        const int r = e / g.nx;
        ix = e - r * g.nx;
        iz = r < NS ? r : g.nz - 1 - (r - NS);
    } else {
        const int c = (e - nud) / g.nz;
        iz = (e - nud) - c * g.nz;
        ix = c < NS ? c : g.nx - 1 - (c - NS);
    }
    const float v = *GP(f + (long long)s * g.fstride + (long long)(iz + g.z0p) * g.ld + ix + g.x0p);
    float* ring = P.ring + sd.ring_off + (long long)(t - P.ring_t0) * P.strip_len;
    *GP(ring + e) = v;
}

// A checkpoint holds the two time levels of the forward field, p^{t_a} (in
// field half ha) and p^{t_a - 1} (the other half), of gridDim.z shots of n
// floats each (halves hs floats apart), laid out [shot][2][n].
//   FP32: both levels, unscaled (exact copies).
//   FP16 / BF16: level 0 = p^{t_a}, level 1 = d = p^{t_a} - p^{t_a - 1}, each
//   scaled by its own absmax (stored = value * SNAP_RANGE / absmax).  Storing
//   the difference keeps the error of the field's time derivative at the
//   storage precision of d; two independently rounded levels would put an
//   error of order (rounding of p) / (p^{t_a} - p^{t_a - 1}), tens of times
//   larger, on it, and the recompute would propagate that as noise.
// 2^14 keeps the largest value well inside FP16's range (65504) and the
// smallest normal FP16 (6.1e-5) at 3.7e-9 of the absmax.
constexpr float SNAP_RANGE = 16384.f;

__device__ __forceinline__ float snap_scale_of(unsigned bits) { const float a = __uint_as_float(bits); return a > 0.f ? a / SNAP_RANGE : 1.f; }

// Largest |p^{t_a}| and |p^{t_a} - p^{t_a-1}| of each shot, as the bits of
// non-negative floats (which order like unsigned integers), in amax[2 s] and
// amax[2 s + 1]; amax must be zero beforehand.
__global__ void k_snap_absmax(const float* __restrict__ f, long long hs, long long n, int ha, unsigned* __restrict__ amax)
{
    const int s = blockIdx.z;
    const float* pa = f + ha * hs + (long long)s * n;
    const float* pb = f + (1 - ha) * hs + (long long)s * n;
    float m0 = 0.f, m1 = 0.f;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float a = pa[i];
        m0 = fmaxf(m0, fabsf(a));
        m1 = fmaxf(m1, fabsf(a - pb[i]));
    }
    for (int o = 16; o > 0; o >>= 1) {
        m0 = fmaxf(m0, __shfl_xor_sync(0xffffffffu, m0, o));
        m1 = fmaxf(m1, __shfl_xor_sync(0xffffffffu, m1, o));
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMax(amax + 2 * s, __float_as_uint(m0));
        atomicMax(amax + 2 * s + 1, __float_as_uint(m1));
    }
}

template <class T> __device__ __forceinline__ T snap_pack(float v);
template <class T> __device__ __forceinline__ float snap_unpack(T q);
template <> __device__ __forceinline__ float snap_pack<float>(float v) { return v; }
template <> __device__ __forceinline__ float snap_unpack<float>(float q) { return q; }
template <> __device__ __forceinline__ __half snap_pack<__half>(float v) { return __float2half_rn(v); }
template <> __device__ __forceinline__ float snap_unpack<__half>(__half q) { return __half2float(q); }
template <> __device__ __forceinline__ __nv_bfloat16 snap_pack<__nv_bfloat16>(float v) { return __float2bfloat16_rn(v); }
template <> __device__ __forceinline__ float snap_unpack<__nv_bfloat16>(__nv_bfloat16 q) { return __bfloat162float(q); }

template <class T>
__global__ void k_snap_store(const float* __restrict__ f, long long hs, long long n, int ha,
                             const unsigned* __restrict__ amax, T* __restrict__ out)
{
    constexpr bool kDelta = sizeof(T) == 2;
    const int s = blockIdx.z;
    const float* pa = f + ha * hs + (long long)s * n;
    const float* pb = f + (1 - ha) * hs + (long long)s * n;
    T* q0 = out + 2LL * s * n;
    T* q1 = q0 + n;
    const float i0 = kDelta ? 1.f / snap_scale_of(amax[2 * s]) : 1.f;
    const float i1 = kDelta ? 1.f / snap_scale_of(amax[2 * s + 1]) : 1.f;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float a = pa[i], b = pb[i];
        q0[i] = snap_pack<T>(a * i0);
        q1[i] = snap_pack<T>(kDelta ? (a - b) * i1 : b);
    }
}

template <class T>
__global__ void k_snap_load(float* __restrict__ f, long long hs, long long n, int ha,
                            const unsigned* __restrict__ amax, const T* __restrict__ in)
{
    constexpr bool kDelta = sizeof(T) == 2;
    const int s = blockIdx.z;
    float* pa = f + ha * hs + (long long)s * n;
    float* pb = f + (1 - ha) * hs + (long long)s * n;
    const T* q0 = in + 2LL * s * n;
    const T* q1 = q0 + n;
    const float s0 = kDelta ? snap_scale_of(amax[2 * s]) : 1.f;
    const float s1 = kDelta ? snap_scale_of(amax[2 * s + 1]) : 1.f;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float a = snap_unpack<T>(q0[i]) * s0;
        pa[i] = a;
        pb[i] = kDelta ? a - snap_unpack<T>(q1[i]) * s1 : snap_unpack<T>(q1[i]);
    }
}

// grad[iz][ix] = 2 / v * sum_s g_s, summed in FP64 in shot order.
__global__ void k_reduce(const float* __restrict__ gacc, const float* __restrict__ vel, double* __restrict__ grad,
                         Geo g, int nshots)
{
    const int ix = blockIdx.x * blockDim.x + threadIdx.x;
    const int iz = blockIdx.y;
    if (ix >= g.nx || iz >= g.nz) return;
    const long long o = (long long)(iz + g.z0p) * g.ld + ix + g.x0p;
    double acc = 0.0;
    for (int s = 0; s < nshots; ++s) acc += (double)gacc[(long long)s * g.fstride + o];
    const long long q = (long long)iz * g.nx + ix;
    grad[q] = 2.0 / (double)vel[q] * acc;
}

__global__ void k_to_float(const double* __restrict__ a, float* __restrict__ b, long long n)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        b[i] = (float)a[i];
}

}  // namespace fwi
