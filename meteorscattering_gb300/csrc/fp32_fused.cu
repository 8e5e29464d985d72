// fp32_fused.cu -- FP32 fused form: one pass over the grid per time step.
//
// Storage: E, H, J and the CPML psi slabs in FP32; the running-DFT sums of the
// Huygens surface in FP64 (the same 24 arrays and layout as the reference's
// output_NTF.dat).  The arithmetic follows the reference's discretisation
// (source/meteor-2.1.cpp:656-1504, source/meteor-fork.cpp:1539-1595) with the
// division by the cell size folded into precomputed FP32 coefficients and FMA
// contraction allowed.
//
// One kernel launch advances one time step.  Each CTA owns a TJ x TK tile of
// (j,k) columns and marches along x (the slowest axis, stride Ny*Nzp), one
// plane per iteration:
//   * the plane's E and H tiles (plus one-cell halos) arrive by TMA
//     (cp.async.bulk.tensor.3d) into a ring of NS shared-memory stages, each
//     guarded by an mbarrier; the producer runs NS-2 planes ahead; J is read
//     from global memory, only in blocks holding plasma (zero elsewhere);
//   * J of the previous step is advanced first (it needs E of this step's
//     start, which is read-only in this pass), then H of this plane (tile plus
//     a low-side halo row and column, which the E update needs), then E;
//   * H and E of the previous plane stay in registers (Hy, Hz, Ex), so each
//     field value is read from DRAM once and written once per step.
// E, H and the H-psi slabs are double-buffered (a pass reads set `par` and
// writes set `par^1`), because neighbouring CTAs read halo cells that another
// CTA writes in the same pass.  J and the E-psi slabs are touched only by
// their owning thread and are updated in place.
#include <cuda.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <map>
#include <algorithm>
#include <mutex>
#include <vector>

#include "fp32.hpp"
#include "incident.cuh"
#include "trail.cuh"

namespace mfdtd {
namespace {

constexpr int TJ = 8, TK = 32;             // tile rows (j) x columns (k)
// One stage is one x plane of the six field components of one parity, a box
// of rows j0-1..j0+TJ and cols k0-4..k0+TK+3 each, loaded by ONE TMA copy:
// the components of a parity are one allocation, [Ex Ey Ez Hx Hy Hz][Nx][Ny][Nzp],
// addressed by a 4-D tensor map.  (Six 3-D copies per plane, one per
// component, kept the producer thread issuing for about 1100 cycles after
// each plane's barrier; it was the last thread to reach the next one.)  The
// H update uses rows j0-1..j0+TJ-1 and cols k0-4..k0+TK-1 of its box.
constexpr int EJ = TJ + 2, EK = TK + 8;
constexpr int HJ = TJ + 1;                 // rows of the new-H plane: j0-1..j0+TJ-1
constexpr int NS = 5;                      // pipeline stages
constexpr int NTHREADS = 320;              // 8 tile warps + halo-row warp + halo-column warp
constexpr int PROD = NTHREADS - 1;         // producer thread (idle lane of the halo-column warp)
constexpr int align128(int b) { return (b + 127) / 128 * 128; }
constexpr int C_B = EJ * EK * 4;           // one component's box (dense in the stage)
constexpr int STAGE_B = align128(6 * C_B);
constexpr int STAGE_TX = 6 * C_B;          // bytes per stage
constexpr int HN_COLS = TK + 1;            // new-H plane: cols k0-1..k0+TK-1
constexpr int HN_B = 3 * HJ * HN_COLS * 4;
constexpr int PF_CAP = 256;                // plasma flags of up to this many planes in shared memory
// two new-H planes (alternating per x plane), NS stage barriers, two poll
// flags, the plasma flags of the CTA's planes
constexpr int SMEM_B = NS * STAGE_B + 2 * align128(HN_B) + NS * 8 + 16 + PF_CAP + 128;  // flags: 3 ints
constexpr double kE0 = 8.85419e-12;

struct Maps {
    CUtensorMap F[2];  // the six components of parity 0 and 1
};

// CPML and auxiliary-line coefficient tables of one simulation, in global
// memory (read on the boundary path only), so that Args stays small enough
// for a batch of simulations to keep their Args in the constant bank.
struct Tables {
    float Bh[2 * kMaxPml], Ahx[2 * kMaxPml], Ahy[2 * kMaxPml], Ahz[2 * kMaxPml];
    float Be[2 * kMaxPml], Aex[2 * kMaxPml], Aey[2 * kMaxPml], Aez[2 * kMaxPml];
    // kappa != 1 derivative terms (1/kappa - 1)/d per slab index
    float Khx[2 * kMaxPml], Khy[2 * kMaxPml], Khz[2 * kMaxPml];
    float Kex[2 * kMaxPml], Key[2 * kMaxPml], Kez[2 * kMaxPml];
    // auxiliary-line CPML (oblique incidence), A pre-divided by the line cell
    float Bh1[2 * kMaxPml], Ah1[2 * kMaxPml], Be1[2 * kMaxPml], Ae1[2 * kMaxPml];
};
// The slab march keeps a copy of the tables in shared memory, after the
// barriers, poll flags and plasma flags.
constexpr int SLAB_TB_OFF = NS * STAGE_B + 2 * align128(HN_B) + align128(NS * 8 + 16 + PF_CAP);
constexpr int SMEM_BS = SLAB_TB_OFF + (int)sizeof(Tables) + 128;

struct Args {
    int Nx, Ny, Nz, Nzp, L, xshift, yshift, zshift;
    int bx1, bx2, by1, by2, bz1, bz2, ntfb, nntf, ssx, ssy, ssz;
    int dopml, doplate, doB0, lk_mode, plate_lo, plate_up, nprobes, tsteps;
    int chunk;           // planes per CTA along x
    // coefficients
    float c1h, chx, chy, chz, c2h;           // c2h/dx ...
    float c1e0, c2e0, cex, cey, cez;         // c2e0/dx ...
    float c1s, c2s, csx, csy, csz;           // sphere (doplate == 2)
    float dtf, c0di;                         // dt, 2*E0*dt
    double platesize;
    const Tables *tb;    // CPML / line tables (global memory)
    float lku[18];       // Lee-Kalluri matrices when nu is uniform over the grid
    int kappa_on;        // kappa != 1: the CPML corrections carry the 1/kappa term
    // oblique incidence: auxiliary line (E in inc[][1], H in inc[][2])
    int oblique, M, ashift, lk_colocated;
    float kr[3], s0, ke[3], kh[3], chl, cel;   // chl = c2h/dl, cel = c2e0/dl
    // The oblique TF/SF corrections made inside the step kernel (1) or by the
    // kernels that follow it (0: k_fp32_tfsf, in a batch k_batch_post).  The
    // running DFT on the Huygens surface always follows the pass: k_fp32_ntf
    // (k_batch_post) copies each step's face values into the DFT ring.
    int obl_inline;
    // Planes [xbeg, xend) are marched by the pass (x-chunks of `chunk` planes
    // from xbeg).  The fast pass leaves the band's x planes to the band
    // kernels (xbeg = L + 1); otherwise 0 and Nx.
    int xbeg, xend;
    // 1: the pass treats CPML and domain-edge cells like interior ones and the
    // band kernels (k_fp32_band_h, k_fp32_band_e) recompute them afterwards;
    // 0: the pass makes the CPML corrections itself (a batch).
    int band;
    // state
    float *E[2][3], *H[2][3], *J[3];
    float *Ph[2][6];     // H psi: xy, xz, yx, yz, zx, zy
    float *Pe[6];        // E psi: xy, xz, yx, yz, zx, zy
    // psi plane strides: y-normal arrays [Nx][2L][Nz], z-normal [Nx][Ny][2L],
    // and the x-normal arrays' slab stride ([2L][Ny][Nz])
    unsigned psi_py, psi_pz, psi_px;
    float *inc[2][4];    // 1-D line: Eyinc, Ezinc, Hyinc, Hzinc
    float *incP[2][4];   // 1-D psi: PeyxI, PezxI, PhyxI, PhzxI
    const float *wq2;    // E0 * wp2^2 per (i,j)
    const float *nu2;    // nu2 per (i,j)
    const float *wq3;    // E0 * wp3^2 per cell (padded layout) or null
    const float *nu3;    // nu3 per cell (padded layout) or null
    const float *G, *G2; // z-Gaussian and its square per k
    const float *lk;     // Lee-Kalluri table (18 per entry)
    const float *src;    // [tsteps][2]
    const double *xc, *yc, *zc;
    const int *tile_order;  // CTA -> tile (ty * ntk + tk): boundary tiles first
    int ntk;                // tiles along k
    // Per (plane, tile): 1 when any cell of the tile's 8 x 32 block in that
    // plane holds plasma (omega_p > 0), else 0.  Elsewhere J is zero and stays
    // zero (its update adds a term proportional to omega_p^2), so the pass
    // neither loads, updates nor stores it there.  Null: plasma everywhere.
    const unsigned char *plasma;
    int ntiles;             // tiles per plane (row length of `plasma`)
    // Work units of the band kernels (Args::band), one per warp at a time:
    // x = i | j << 16; y = first cell | count << 16 | band-list flag << 24.
    const int2 *band_units;
    int n_band_units;
    double *ntf[24];
    // Running-DFT ring (k_fp32_ntf's layout) and split phase table
    // (k_fp32_ntf_flush); a batch member's are set when it joins its batch.
    float *ntf_ring;
    const float4 *phase4;
    double *probe;       // [6][tsteps][nprobes]
    const int *probe_ijk;
    float *slE, *slH;
    unsigned int *err;   // bit 0: a TMA wait ran out
};

// ---------------------------------------------------------------------------
// PTX helpers: mbarrier and TMA
__device__ __forceinline__ unsigned smem_u32(const void *p) {
    return (unsigned)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t *bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arm(uint64_t *bar, unsigned tx) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(tx)
                 : "memory");
}
__device__ __forceinline__ bool mbar_test(uint64_t *bar, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
__device__ __forceinline__ uint64_t globaltimer() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
// Bounded wait: gives up after ~2 s of wall time.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, unsigned parity) {
    if (mbar_test(bar, parity)) return true;
    const uint64_t t0 = globaltimer();
    for (;;) {
        if (mbar_test(bar, parity)) return true;
        if (globaltimer() - t0 > 2000000000ull) return false;
    }
}
__device__ __forceinline__ void tma4(void *dst, const CUtensorMap *map, int c0, int c1, int c2, int c3,
                                     uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, "
        "%3, %4, %5}], [%6];" ::"r"(smem_u32(dst)),
        "l"((uint64_t)map), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(smem_u32(bar))
        : "memory");
}

__device__ __forceinline__ int hslab(int n, int N, int L, int shift) {
    if (n < L) return n;
    if (n >= N - L - 1 && n < N - 1) return n - shift;
    return -1;
}
__device__ __forceinline__ int eslab(int n, int N, int L, int shift) {
    if (n >= 1 && n < L + 1) return n - 1;
    if (n >= N - L - 1 && n < N - 1) return n - shift;
    return -1;
}

// Views of one stage.
struct Stage {
    float *e[3], *h[3];
};
__device__ __forceinline__ Stage stage_at(unsigned char *base) {
    Stage s;
    for (int c = 0; c < 3; c++) {
        s.e[c] = (float *)(base + c * C_B);
        s.h[c] = (float *)(base + (3 + c) * C_B);
    }
    return s;
}
// Box element at (j,k) relative to the tile origin: row j - (j0-1), col k - (k0-4)
#define EIDX(dj, dk) (((dj) + 1) * EK + (dk) + 4)
#define HIDX(dj, dk) EIDX(dj, dk)
#define HN(c, dj, dk) hn[((c) * HJ + (dj) + 1) * HN_COLS + (dk) + 1]

struct HVal {
    float x, y, z;
};

__device__ __forceinline__ bool hits(int lo, int hi, int v) { return v >= lo && v <= hi; }

// ---- oblique incidence (extended inputs) ----------------------------------
// Same construction as the FP64 plain form: a node with doubled coordinates P
// sees the auxiliary line at s = kr . P/2 + s0; every curl term whose
// neighbour lies across the TF/SF box surface gets the neighbour's incident
// value.  H targets use the line's E of this pass's start; E targets use the
// line's H of this step, computed here from the start-of-pass line (the line
// itself is advanced by the first CTA into the other buffer).
__device__ __forceinline__ bool obl_shell(const Args &a, int i, int j, int k) {
    return i >= a.bx1 - 1 && i <= a.bx2 && j >= a.by1 - 1 && j <= a.by2 && k >= a.bz1 - 1 &&
           k <= a.bz2 &&
           !(i > a.bx1 && i < a.bx2 - 2 && j > a.by1 && j < a.by2 - 2 && k > a.bz1 && k < a.bz2 - 2);
}
template <int PAR>
__device__ __forceinline__ float obl_e_at(const Args &a, float s) {
    const float *e = a.inc[PAR][1];
    const float fl = floorf(s);
    const int n = (int)fl;
    return __fadd_rn(e[n], __fmul_rn(__fsub_rn(s, fl), __fsub_rn(e[n + 1], e[n])));
}
template <int PAR>
__device__ __forceinline__ float obl_h_new_at(const Args &a, float s) {
    const float *e = a.inc[PAR][1], *h = a.inc[PAR][2];
    const float fl = floorf(s);
    const int n = (int)fl;
    const float h0 = __fsub_rn(__fmul_rn(a.c1h, h[n]), __fmul_rn(a.chl, __fsub_rn(e[n + 1], e[n])));
    const float h1 = __fsub_rn(__fmul_rn(a.c1h, h[n + 1]), __fmul_rn(a.chl, __fsub_rn(e[n + 2], e[n + 1])));
    return __fadd_rn(h0, __fmul_rn(__fsub_rn(s, fl), __fsub_rn(h1, h0)));
}
// Crossing term along axis AX for component C of E (IS_E) or H at cell
// (i,j,k), already scaled by c2/d_AX.  Along one axis a node type crosses the
// box surface at two indices only (H: b1-1 and b2-1; E: b1 and b2-1), and only
// where its coordinates along the other two axes lie inside the box; the
// neighbour across the surface is the third component.  Same terms as the
// generic construction (sign = curl sign x side x (T - Tn)).
template <int PAR, bool IS_E, int C, int AX>
__device__ __forceinline__ float obl_axis(const Args &a, int i, int j, int k) {
    constexpr int Q = 3 - C - AX;                                     // neighbour component
    constexpr int SG = (AX == (C + 1) % 3) ? (IS_E ? 1 : -1) : (IS_E ? -1 : 1);
    const int idx[3] = {i, j, k};
    const int b1[3] = {a.bx1, a.by1, a.bz1}, b2[3] = {a.bx2, a.by2, a.bz2};
    const int n = idx[AX];
    int nb;      // neighbour index along AX
    float sgn;
    if (IS_E) {
        if (n == b1[AX]) { nb = n - 1; sgn = (float)-SG; }
        else if (n == b2[AX] - 1) { nb = n; sgn = (float)SG; }
        else return 0.f;
    } else {
        if (n == b1[AX] - 1) { nb = n + 1; sgn = (float)-SG; }
        else if (n == b2[AX] - 1) { nb = n; sgn = (float)SG; }
        else return 0.f;
    }
    // doubled coordinates of the neighbour: E comp Q is staggered along Q only,
    // H comp Q along the two axes other than Q
    int P[3];
#pragma unroll
    for (int d = 0; d < 3; d++) {
        const int st = IS_E ? (d != Q) : (d == Q);  // neighbour staggering
        const int tst = IS_E ? (d == C) : (d != C); // target staggering
        P[d] = d == AX ? 2 * nb + st : 2 * idx[d] + tst;
        if (d != AX && (P[d] < 2 * b1[d] || P[d] > 2 * (b2[d] - 1))) return 0.f;
    }
    // (explicitly rounded operations: the corrections come out the same bits
    // in every kernel that inlines them, whatever the compiler contracts)
    const float sp = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(a.kr[0], 0.5f * P[0]), __fmul_rn(a.kr[1], 0.5f * P[1])),
                                         __fmul_rn(a.kr[2], 0.5f * P[2])),
                               a.s0);
    const float inc = IS_E ? __fmul_rn(a.kh[Q], obl_h_new_at<PAR>(a, __fsub_rn(sp, 0.5f)))
                           : __fmul_rn(a.ke[Q], obl_e_at<PAR>(a, sp));
    const float cd = IS_E ? (AX == 0 ? a.cex : AX == 1 ? a.cey : a.cez)
                          : (AX == 0 ? a.chx : AX == 1 ? a.chy : a.chz);
    return __fmul_rn(__fmul_rn(sgn, inc), cd);
}
template <int PAR, bool IS_E, int C>
__device__ __forceinline__ float obl_corr(const Args &a, int i, int j, int k) {
    return __fadd_rn(obl_axis<PAR, IS_E, C, (C + 1) % 3>(a, i, j, k), obl_axis<PAR, IS_E, C, (C + 2) % 3>(a, i, j, k));
}

// Per-tile facts that are uniform across the CTA.
struct TileInfo {
    bool clean;   // no y/z CPML, TF/SF, NTF, slice, plate or domain-edge rows/columns
    bool tf_in;   // (clean tiles) the whole tile lies inside the TF/SF box in j and k
};


__device__ TileInfo classify(const Args &a, int j0, int k0, int record) {
    TileInfo ti;
    const int jlo = j0 - 1, jhi = j0 + TJ, klo = k0 - 1, khi = k0 + TK;
    const int Ny = a.Ny, Nz = a.Nz, L = a.dopml ? a.L : 0;
    bool c = a.doplate == 0;
    if (!a.band) {  // (with the band kernels, CPML and edge rows are fixed after the pass)
        c = c && jlo >= L + 1 && jhi <= Ny - L - 2 && klo >= L + 1 && khi <= Nz - L - 2;
        c = c && jlo >= 1 && jhi <= Ny - 2 && klo >= 1 && khi <= Nz - 2;
    }
    auto clear = [&](int vy, int vz) { return !hits(jlo, jhi, vy) && !hits(klo, khi, vz); };
    if (!a.oblique || a.obl_inline)  // TF/SF rows, when the corrections are made here
        c = c && clear(a.by1 - 1, a.bz1 - 1) && clear(a.by1, a.bz1) && clear(a.by2 - 1, a.bz2 - 1) &&
            clear(a.by2, a.bz2);
    // slices are written on record steps only
    c = c && !(record && (hits(jlo, jhi, a.ssy) || hits(klo, khi, a.ssz)));
    ti.clean = c;
    ti.tf_in = jlo > a.by1 && jhi < a.by2 - 1 && klo > a.bz1 && khi < a.bz2 - 1;
    return ti;
}

// Where h_cell reads the old fields of a cell and of its +j, +k and +i
// neighbours: the stage boxes in shared memory (the pass), or the values the
// CPML band kernels load before the update (PreSrcView).  A neighbour is used
// only where the update needs it.
struct StageSrc {
    const Stage &s, &s1;
    int dj, dk;
    __device__ __forceinline__ float h(int c) const { return s.h[c][HIDX(dj, dk)]; }
    __device__ __forceinline__ float e(int c) const { return s.e[c][EIDX(dj, dk)]; }
    __device__ __forceinline__ float ej(int c) const { return s.e[c][EIDX(dj + 1, dk)]; }
    __device__ __forceinline__ float ek(int c) const { return s.e[c][EIDX(dj, dk + 1)]; }
    __device__ __forceinline__ float ei(int c) const { return s1.e[c][EIDX(dj, dk)]; }
};

// H half-step of one cell (source/meteor-2.1.cpp:656-937 in FP32), reading
// the old fields through `src`.  Components outside their update domain keep
// their old value.  `store_psi` is false for halo cells computed on behalf of
// a neighbouring tile; `pml` says whether the CPML corrections are made here
// (the pass leaves them to the band kernels).  In a clean tile only the
// x-dependent special cases (uniform across the CTA) can occur.  With HOIST
// the cell's psi values are all loaded before its first update, so that the
// loads overlap (a psi load placed after another component's psi store cannot
// be moved above it: the two may alias); the band kernels use it, the pass
// does not (the registers it holds made the pass spill).
// LEAN (the CPML slab march): the TF/SF corrections are made after the pass
// (oblique incidence) and there is no plate or sphere, so that code is not
// compiled in.
template <int PAR, bool CLEAN, bool HOIST = false, bool LEAN = false, class Src>
__device__ __forceinline__ HVal h_cell(const Args &a, int i, int j, int k, const Src &src, bool store_psi,
                                       bool want_y, bool want_z, bool tf_in, bool pml) {
    const int Nx = a.Nx, Ny = a.Ny, Nz = a.Nz, L = a.L;
    HVal o;
    o.x = src.h(0);
    o.y = src.h(1);
    o.z = src.h(2);
    const float ex = src.e(0), ey = src.e(1), ez = src.e(2);
    const bool xin = i < Nx - 1;
    const int sx = pml ? hslab(i, Nx, L, a.xshift) : -1;
    const bool inbx = i >= a.bx1 && i < a.bx2;
    const bool inby = CLEAN ? tf_in : (j >= a.by1 && j < a.by2);
    const bool inbz = CLEAN ? tf_in : (k >= a.bz1 && k < a.bz2);
    float pp[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};  // HOIST: Ph[PAR][0..5] of this cell
    if (HOIST && pml) {
        const int sy = CLEAN ? -1 : hslab(j, Ny, L, a.yshift), sz = CLEAN ? -1 : hslab(k, Nz, L, a.zshift);
        const bool ux = CLEAN || (j < Ny - 1 && k < Nz - 1);
        const bool uy = want_y && xin && (CLEAN || k < Nz - 1);
        const bool uz = want_z && xin && (CLEAN || j < Ny - 1);
        // (indices of absent slabs clamped to 0: never used)
        const size_t oy = ((size_t)i * (2 * L) + max(sy, 0)) * Nz + k,
                     oz = ((size_t)i * Ny + j) * (2 * L) + max(sz, 0), ox = ((size_t)max(sx, 0) * Ny + j) * Nz + k;
        if (ux && sy >= 0) pp[0] = a.Ph[PAR][0][oy];
        if (ux && sz >= 0) pp[1] = a.Ph[PAR][1][oz];
        if (uy && sx >= 0) pp[2] = a.Ph[PAR][2][ox];
        if (uy && sz >= 0) pp[3] = a.Ph[PAR][3][oz];
        if (uz && sx >= 0) pp[4] = a.Ph[PAR][4][ox];
        if (uz && sy >= 0) pp[5] = a.Ph[PAR][5][oy];
    }
    if (CLEAN || (j < Ny - 1 && k < Nz - 1)) {
        const float dEz = src.ej(2) - ez;
        const float dEy = src.ek(1) - ey;
        float h = a.c1h * o.x - (a.chy * dEz - a.chz * dEy);
        if (!CLEAN) {
            if (LEAN) {
            } else if (!a.oblique) {
                if (inbx && inbz) {
                    const float ezi = a.inc[PAR][1][i];
                    if (j == a.by1 - 1) h += a.chy * ezi;
                    if (j == a.by2 - 1) h -= a.chy * ezi;
                }
                if (inbx && inby) {
                    const float eyi = a.inc[PAR][0][i];
                    if (k == a.bz1 - 1) h -= a.chz * eyi;
                    if (k == a.bz2 - 1) h += a.chz * eyi;
                }
            } else if (a.obl_inline && obl_shell(a, i, j, k)) {
                h += obl_corr<PAR, false, 0>(a, i, j, k);
            }
            if (pml) {
                const int sy = hslab(j, Ny, L, a.yshift);
                if (sy >= 0) {
                    const size_t o2 = ((size_t)i * (2 * L) + sy) * Nz + k;
                    const float p = a.tb->Bh[sy] * (HOIST ? pp[0] : a.Ph[PAR][0][o2]) + a.tb->Ahy[sy] * dEz;
                    if (store_psi) a.Ph[PAR ^ 1][0][o2] = p;
                    h -= a.c2h * p;
                    if (a.kappa_on) h -= a.c2h * (a.tb->Khy[sy] * dEz);
                }
                const int sz = hslab(k, Nz, L, a.zshift);
                if (sz >= 0) {
                    const size_t o2 = ((size_t)i * Ny + j) * (2 * L) + sz;
                    const float p = a.tb->Bh[sz] * (HOIST ? pp[1] : a.Ph[PAR][1][o2]) + a.tb->Ahz[sz] * dEy;
                    if (store_psi) a.Ph[PAR ^ 1][1][o2] = p;
                    h += a.c2h * p;
                    if (a.kappa_on) h += a.c2h * (a.tb->Khz[sz] * dEy);
                }
            }
        }
        o.x = h;
    }
    if (want_y && xin && (CLEAN || k < Nz - 1)) {
        const float dEx = src.ek(0) - ex;
        const float dEz = src.ei(2) - ez;
        float h = a.c1h * o.y - (a.chz * dEx - a.chx * dEz);
        if (LEAN) {
        } else if (!a.oblique) {
            if (inby && inbz) {
                if (i == a.bx1 - 1) h -= a.chx * a.inc[PAR][1][a.bx1];
                if (i == a.bx2 - 1) h += a.chx * a.inc[PAR][1][a.bx2 - 1];
            }
        } else if (a.obl_inline && obl_shell(a, i, j, k)) {
            h += obl_corr<PAR, false, 1>(a, i, j, k);
        }
        if (sx >= 0) {
            const size_t o2 = ((size_t)sx * Ny + j) * Nz + k;
            const float p = a.tb->Bh[sx] * (HOIST ? pp[2] : a.Ph[PAR][2][o2]) + a.tb->Ahx[sx] * dEz;
            if (store_psi) a.Ph[PAR ^ 1][2][o2] = p;
            h += a.c2h * p;
            if (a.kappa_on) h += a.c2h * (a.tb->Khx[sx] * dEz);
        }
        if (!CLEAN && pml) {
            const int sz = hslab(k, Nz, L, a.zshift);
            if (sz >= 0) {
                const size_t o2 = ((size_t)i * Ny + j) * (2 * L) + sz;
                const float p = a.tb->Bh[sz] * (HOIST ? pp[3] : a.Ph[PAR][3][o2]) + a.tb->Ahz[sz] * dEx;
                if (store_psi) a.Ph[PAR ^ 1][3][o2] = p;
                h -= a.c2h * p;
                if (a.kappa_on) h -= a.c2h * (a.tb->Khz[sz] * dEx);
            }
        }
        o.y = h;
    }
    if (want_z && xin && (CLEAN || j < Ny - 1)) {
        const float dEy = src.ei(1) - ey;
        const float dEx = src.ej(0) - ex;
        float h = a.c1h * o.z - (a.chx * dEy - a.chy * dEx);
        if (LEAN) {
        } else if (!a.oblique) {
            if (inby && inbz) {
                if (i == a.bx1 - 1) h += a.chx * a.inc[PAR][0][a.bx1];
                if (i == a.bx2 - 1) h -= a.chx * a.inc[PAR][0][a.bx2 - 1];
            }
        } else if (a.obl_inline && obl_shell(a, i, j, k)) {
            h += obl_corr<PAR, false, 2>(a, i, j, k);
        }
        if (sx >= 0) {
            const size_t o2 = ((size_t)sx * Ny + j) * Nz + k;
            const float p = a.tb->Bh[sx] * (HOIST ? pp[4] : a.Ph[PAR][4][o2]) + a.tb->Ahx[sx] * dEy;
            if (store_psi) a.Ph[PAR ^ 1][4][o2] = p;
            h -= a.c2h * p;
            if (a.kappa_on) h -= a.c2h * (a.tb->Khx[sx] * dEy);
        }
        if (!CLEAN && pml) {
            const int sy = hslab(j, Ny, L, a.yshift);
            if (sy >= 0) {
                const size_t o2 = ((size_t)i * (2 * L) + sy) * Nz + k;
                const float p = a.tb->Bh[sy] * (HOIST ? pp[5] : a.Ph[PAR][5][o2]) + a.tb->Ahy[sy] * dEx;
                if (store_psi) a.Ph[PAR ^ 1][5][o2] = p;
                h += a.c2h * p;
                if (a.kappa_on) h += a.c2h * (a.tb->Khy[sy] * dEx);
            }
        }
        o.z = h;
    }
    return o;
}

// Incident-line H value of this step at index i (the 1-D update of
// source/meteor-2.1.cpp:833, 892 without the +x CPML term, which never
// reaches the TF/SF planes).
template <int PAR>
__device__ __forceinline__ float hyinc_new(const Args &a, int i) {
    const float *ez = a.inc[PAR][1];
    return a.c1h * a.inc[PAR][2][i] + a.chx * (ez[i + 1] - ez[i]);
}
template <int PAR>
__device__ __forceinline__ float hzinc_new(const Args &a, int i) {
    const float *ey = a.inc[PAR][0];
    return a.c1h * a.inc[PAR][3][i] - a.chx * (ey[i + 1] - ey[i]);
}

// Where e_cell reads the new H of the cell's -j, -k and -i neighbours: the
// new-H planes in shared memory and the previous plane's values kept in
// registers (the pass), or the values the CPML band kernels load before the
// update (PreHSrcView).
struct StageHSrc {
    const float *hn;
    int dj, dk;
    float hy_prev, hz_prev;
    __device__ __forceinline__ float hj(int c) const { return HN(c, dj - 1, dk); }
    __device__ __forceinline__ float hk(int c) const { return HN(c, dj, dk - 1); }
    __device__ __forceinline__ float hyi() const { return hy_prev; }
    __device__ __forceinline__ float hzi() const { return hz_prev; }
};

struct EVal {
    float x, y, z, z_slice;  // z_slice: Ez before its CPML corrections (the slice value)
};

// E half-step of one cell (source/meteor-2.1.cpp:1020-1374 in FP32): the old
// E (ex, ey, ez), the cell's new H (hv), the neighbours' new H through `hs`,
// the current (jx, jy, jz).  `pml` as in h_cell.
template <int PAR, bool CLEAN, bool HOIST = false, bool LEAN = false, class HS>
__device__ __forceinline__ EVal e_cell(const Args &a, int i, int j, int k, float ex, float ey, float ez, const HVal &hv,
                                       const HS &hs, float jx, float jy, float jz, bool tf_in, bool pml) {
    const int Nx = a.Nx, Ny = a.Ny, Nz = a.Nz, L = a.L;
    bool sphere = false;
    if (!CLEAN && !LEAN && a.doplate == 2) {
        const double x = a.xc[i], y = a.yc[j], z = a.zc[k];
        sphere = sqrt(x * x + y * y + z * z) < a.platesize;
    }
    const float c1 = sphere ? a.c1s : a.c1e0, c2 = sphere ? a.c2s : a.c2e0;
    const float cx = sphere ? a.csx : a.cex, cy = sphere ? a.csy : a.cey,
                cz = sphere ? a.csz : a.cez;
    const bool plate_row = !CLEAN && !LEAN && a.doplate == 1 && i == a.ssx;
    const int sxe = pml ? eslab(i, Nx, L, a.xshift) : -1;
    const bool inby = CLEAN ? tf_in : (j >= a.by1 && j < a.by2);
    const bool inbz = CLEAN ? tf_in : (k >= a.bz1 && k < a.bz2);
    float pp[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};  // HOIST (see h_cell): Pe[0..5] of this cell
    if (HOIST && pml) {
        const int sy = CLEAN ? -1 : eslab(j, Ny, L, a.yshift), sz = CLEAN ? -1 : eslab(k, Nz, L, a.zshift);
        const bool ux = i < Nx - 1 && (CLEAN || (j >= 1 && j < Ny - 1 && k >= 1 && k < Nz - 1));
        const bool uy = i >= 1 && i < Nx - 1 && (CLEAN || k >= 1);
        const bool uz = i >= 1 && i < Nx - 1 && (CLEAN || j >= 1);
        const bool xp = sxe >= 0 && (CLEAN || (j < Ny - 1 && k < Nz - 1));
        // (indices of absent slabs clamped to 0: never used)
        const size_t oy = ((size_t)i * (2 * L) + max(sy, 0)) * Nz + k,
                     oz = ((size_t)i * Ny + j) * (2 * L) + max(sz, 0), ox = ((size_t)max(sxe, 0) * Ny + j) * Nz + k;
        if (ux && sy >= 0) pp[0] = a.Pe[0][oy];
        if (ux && sz >= 0) pp[1] = a.Pe[1][oz];
        if (uy && xp) pp[2] = a.Pe[2][ox];
        if (uy && sz >= 0 && j < Ny - 1) pp[3] = a.Pe[3][oz];
        if (uz && xp) pp[4] = a.Pe[4][ox];
        if (uz && sy >= 0 && k < Nz - 1) pp[5] = a.Pe[5][oy];
    }
    // Ex
    if (i < Nx - 1 && (CLEAN || (j >= 1 && j < Ny - 1 && k >= 1 && k < Nz - 1))) {
        const float dHz = hv.z - hs.hj(2);
        const float dHy = hv.y - hs.hk(1);
        float e = c1 * ex + (cy * dHz - cz * dHy) - c2 * jx;
        if (!CLEAN) {
            if (LEAN) {
            } else if (a.oblique) {
                if (a.obl_inline && obl_shell(a, i, j, k)) e += obl_corr<PAR, true, 0>(a, i, j, k);
            } else if (i >= a.bx1 && i < a.bx2 - 1) {
                if (inby) {
                    if (k == a.bz1) e += a.cez * hyinc_new<PAR>(a, i);
                    if (k == a.bz2) e -= a.cez * hyinc_new<PAR>(a, i);
                }
                if (inbz) {
                    if (j == a.by1) e -= a.cey * hzinc_new<PAR>(a, i);
                    if (j == a.by2) e += a.cey * hzinc_new<PAR>(a, i);
                }
            }
            if (pml) {
                const int sy = eslab(j, Ny, L, a.yshift);
                if (sy >= 0) {
                    const size_t o2 = ((size_t)i * (2 * L) + sy) * Nz + k;
                    const float p = a.tb->Be[sy] * (HOIST ? pp[0] : a.Pe[0][o2]) + a.tb->Aey[sy] * dHz;
                    a.Pe[0][o2] = p;
                    e += a.c2e0 * p;
                    if (a.kappa_on) e += a.c2e0 * (a.tb->Key[sy] * dHz);
                }
                const int sz = eslab(k, Nz, L, a.zshift);
                if (sz >= 0) {
                    const size_t o2 = ((size_t)i * Ny + j) * (2 * L) + sz;
                    const float p = a.tb->Be[sz] * (HOIST ? pp[1] : a.Pe[1][o2]) + a.tb->Aez[sz] * dHy;
                    a.Pe[1][o2] = p;
                    e -= a.c2e0 * p;
                    if (a.kappa_on) e -= a.c2e0 * (a.tb->Kez[sz] * dHy);
                }
            }
        }
        ex = e;
    }
    // Ey
    if (i >= 1 && i < Nx - 1 && (CLEAN || k >= 1)) {
        const float dHx = hv.x - hs.hk(0);
        const float dHz = hv.z - hs.hzi();
        float e = c1 * ey + (cz * dHx - cx * dHz) - c2 * jy;
        if (LEAN) {
        } else if (!a.oblique) {
            if (inby && inbz) {
                if (i == a.bx1) e += a.cex * hzinc_new<PAR>(a, a.bx1 - 1);
                if (i == a.bx2 - 1) e -= a.cex * hzinc_new<PAR>(a, a.bx2 - 1);
            }
        } else if (a.obl_inline && obl_shell(a, i, j, k)) {
            e += obl_corr<PAR, true, 1>(a, i, j, k);
        }
        if (sxe >= 0) {
            float p = 0.f;
            if (CLEAN || (j < Ny - 1 && k < Nz - 1)) {
                const size_t o2 = ((size_t)sxe * Ny + j) * Nz + k;
                p = a.tb->Be[sxe] * (HOIST ? pp[2] : a.Pe[2][o2]) + a.tb->Aex[sxe] * dHz;
                a.Pe[2][o2] = p;
            }
            e -= a.c2e0 * p;
            if (a.kappa_on) e -= a.c2e0 * (a.tb->Kex[sxe] * dHz);
        }
        if (!CLEAN && pml) {
            const int sz = eslab(k, Nz, L, a.zshift);
            if (sz >= 0) {
                float p = 0.f;
                if (j < Ny - 1) {
                    const size_t o2 = ((size_t)i * Ny + j) * (2 * L) + sz;
                    p = a.tb->Be[sz] * (HOIST ? pp[3] : a.Pe[3][o2]) + a.tb->Aez[sz] * dHx;
                    a.Pe[3][o2] = p;
                }
                e += a.c2e0 * p;
                if (a.kappa_on) e += a.c2e0 * (a.tb->Kez[sz] * dHx);
            }
        }
        ey = e;
    }
    if (plate_row && j >= a.plate_lo && j < a.plate_up - 1 && k >= a.plate_lo && k < a.plate_up)
        ey = 0.f;
    // Ez
    const bool ez_plate = plate_row && j >= a.plate_lo && j < a.plate_up &&
                          k >= a.plate_lo && k < a.plate_up - 1;
    float ez_slice = ez;
    if (i >= 1 && i < Nx - 1 && (CLEAN || j >= 1)) {
        const float dHy = hv.y - hs.hyi();
        const float dHx = hv.x - hs.hj(0);
        float e = c1 * ez + (cx * dHy - cy * dHx) - c2 * jz;
        if (LEAN) {
        } else if (!a.oblique) {
            if (inby && inbz) {
                if (i == a.bx1) e -= a.cex * hyinc_new<PAR>(a, a.bx1 - 1);
                if (i == a.bx2 - 1) e += a.cex * hyinc_new<PAR>(a, a.bx2 - 1);
            }
        } else if (a.obl_inline && obl_shell(a, i, j, k)) {
            e += obl_corr<PAR, true, 2>(a, i, j, k);
        }
        if (ez_plate) e = 0.f;
        ez_slice = e;
        if (sxe >= 0) {
            float p = 0.f;
            if (CLEAN || (j < Ny - 1 && k < Nz - 1)) {
                const size_t o2 = ((size_t)sxe * Ny + j) * Nz + k;
                p = a.tb->Be[sxe] * (HOIST ? pp[4] : a.Pe[4][o2]) + a.tb->Aex[sxe] * dHy;
                a.Pe[4][o2] = p;
            }
            e += a.c2e0 * p;
            if (a.kappa_on) e += a.c2e0 * (a.tb->Kex[sxe] * dHy);
        }
        if (!CLEAN && pml) {
            const int sy = eslab(j, Ny, L, a.yshift);
            if (sy >= 0 && k < Nz - 1) {
                const size_t o2 = ((size_t)i * (2 * L) + sy) * Nz + k;
                const float p = a.tb->Be[sy] * (HOIST ? pp[5] : a.Pe[5][o2]) + a.tb->Aey[sy] * dHx;
                a.Pe[5][o2] = p;
                e -= a.c2e0 * p;
                if (a.kappa_on) e -= a.c2e0 * (a.tb->Key[sy] * dHx);
            }
        }
        ez = e;
    } else if (ez_plate) {
        ez = 0.f;
        ez_slice = 0.f;
    }
    return EVal{ex, ey, ez, ez_slice};
}

// ---- the slab march's CPML cell updates ------------------------------------
// h_cell / e_cell with the CPML corrections (pml), without the TF/SF, plate,
// sphere, DFT and slice code (LEAN), in a form for the slab march: what does
// not change along x is computed once per thread (SlabCell: slab indices,
// domain-edge flags, 32-bit psi offsets at plane 0), the CPML coefficient
// tables are read from a shared-memory copy, and the cell's psi values are
// loaded before its first update.  The expression trees are h_cell's and
// e_cell's, so the results are the same.
struct SlabCell {
    int syh, szh, sye, sze;         // H and E slab indices along y and z (-1: none)
    bool jn, kn, j1, k1;            // j < Ny-1, k < Nz-1, j >= 1, k >= 1
    unsigned oyh, oye, ozh, oze;    // y- and z-normal psi offsets at plane 0
    unsigned ox;                    // x-normal psi offset within a slab plane
    // the y- and z-normal CPML coefficients of the cell (B, A, K of H and E),
    // read once per item in the axis-specialized marches (slab_coef)
    float bhy, ahy, khy, bey, aey, key, bhz, ahz, khz, bez, aez, kez;
};
__device__ __forceinline__ SlabCell slab_cell(const Args &a, int j, int k) {
    SlabCell c;
    const int L = a.L;
    c.syh = hslab(j, a.Ny, L, a.yshift);
    c.szh = hslab(k, a.Nz, L, a.zshift);
    c.sye = eslab(j, a.Ny, L, a.yshift);
    c.sze = eslab(k, a.Nz, L, a.zshift);
    c.jn = j < a.Ny - 1;
    c.kn = k < a.Nz - 1;
    c.j1 = j >= 1;
    c.k1 = k >= 1;
    c.oyh = (unsigned)max(c.syh, 0) * a.Nz + k;
    c.oye = (unsigned)max(c.sye, 0) * a.Nz + k;
    c.ozh = (unsigned)j * (2 * L) + max(c.szh, 0);
    c.oze = (unsigned)j * (2 * L) + max(c.sze, 0);
    c.ox = (unsigned)j * a.Nz + k;
    return c;
}

// A slab-march tile whose cells and halos all lie inside the grid's y
// interior (rows [w, Ny - w - 1], w = L + 1: no y slab, no y face) or its z
// interior marches with that axis's slab indices and face flags as
// constants: YZ bit 0 keeps the y ones, bit 1 the z ones.  The compiler then
// drops that axis's psi terms and tests from the cell updates; the arithmetic
// of the terms that remain is unchanged.
template <int YZ>
__device__ __forceinline__ SlabCell slab_view(SlabCell c) {
    if constexpr (!(YZ & 1)) {
        c.syh = -1;
        c.sye = -1;
        c.jn = true;
        c.j1 = true;
    }
    if constexpr (!(YZ & 2)) {
        c.szh = -1;
        c.sze = -1;
        c.kn = true;
        c.k1 = true;
    }
    return c;
}

// In a march specialized to one axis (YZ 0, 1, 2) the cell's CPML
// coefficients along the axis it keeps are loaded from the shared-memory
// tables once per item instead of on every plane (the plane loop's barriers
// and fences keep the compiler from hoisting those loads itself).  The
// general march (YZ 3) reads them at the point of use.
template <int YZ>
__device__ __forceinline__ SlabCell slab_coef(SlabCell c, const Tables &T) {
    if constexpr (YZ == 1) {
        const int h = max(c.syh, 0), e = max(c.sye, 0);
        c.bhy = T.Bh[h];
        c.ahy = T.Ahy[h];
        c.khy = T.Khy[h];
        c.bey = T.Be[e];
        c.aey = T.Aey[e];
        c.key = T.Key[e];
    }
    if constexpr (YZ == 2) {
        const int h = max(c.szh, 0), e = max(c.sze, 0);
        c.bhz = T.Bh[h];
        c.ahz = T.Ahz[h];
        c.khz = T.Khz[h];
        c.bez = T.Be[e];
        c.aez = T.Aez[e];
        c.kez = T.Kez[e];
    }
    return c;
}

// The six psi values of a cell's H (or E) update on plane i, as h_slab (or
// e_slab) uses them; zero where unused.  The slab march loads them one plane
// ahead, so that their latency overlaps the previous plane's work.
struct Psi6 {
    float p0, p1, p2, p3, p4, p5;
};
template <int PAR>
__device__ __forceinline__ Psi6 h_slab_psi(const Args &a, int i, int sxh, const SlabCell &sc, bool want_y,
                                           bool want_z) {
    const bool xin = i < a.Nx - 1;
    const unsigned PY = a.psi_py, PZ = a.psi_pz, PX = a.psi_px;
    const bool ux = sc.jn && sc.kn, uy = want_y && xin && sc.kn, uz = want_z && xin && sc.jn;
    const unsigned oy = sc.oyh + (unsigned)i * PY, oz = sc.ozh + (unsigned)i * PZ,
                   ox = (unsigned)max(sxh, 0) * PX + sc.ox;
    float *const *R = a.Ph[PAR];
    Psi6 q{0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    if (ux && sc.syh >= 0) q.p0 = R[0][oy];
    if (ux && sc.szh >= 0) q.p1 = R[1][oz];
    if (uy && sxh >= 0) q.p2 = R[2][ox];
    if (uy && sc.szh >= 0) q.p3 = R[3][oz];
    if (uz && sxh >= 0) q.p4 = R[4][ox];
    if (uz && sc.syh >= 0) q.p5 = R[5][oy];
    return q;
}
__device__ __forceinline__ Psi6 e_slab_psi(const Args &a, int i, int sxe, const SlabCell &sc) {
    const bool iy = i >= 1 && i < a.Nx - 1;
    const bool ux = i < a.Nx - 1 && sc.j1 && sc.jn && sc.k1 && sc.kn, uy = iy && sc.k1, uz = iy && sc.j1;
    const bool xp = sxe >= 0 && sc.jn && sc.kn;
    const unsigned PY = a.psi_py, PZ = a.psi_pz, PX = a.psi_px;
    const unsigned oy = sc.oye + (unsigned)i * PY, oz = sc.oze + (unsigned)i * PZ,
                   ox = (unsigned)max(sxe, 0) * PX + sc.ox;
    float *const *Pe = a.Pe;
    Psi6 q{0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    if (ux && sc.sye >= 0) q.p0 = Pe[0][oy];
    if (ux && sc.sze >= 0) q.p1 = Pe[1][oz];
    if (uy && xp) q.p2 = Pe[2][ox];
    if (uy && sc.sze >= 0 && sc.jn) q.p3 = Pe[3][oz];
    if (uz && xp) q.p4 = Pe[4][ox];
    if (uz && sc.sye >= 0 && sc.kn) q.p5 = Pe[5][oy];
    return q;
}

template <int PAR, int YZ, class Src>
__device__ __forceinline__ HVal h_slab(const Args &a, const Tables &T, int i, int sxh, const Src &src,
                                       const SlabCell &sc, bool store_psi, bool want_y, bool want_z,
                                       const Psi6 &ps) {
    HVal o;
    o.x = src.h(0);
    o.y = src.h(1);
    o.z = src.h(2);
    const float ex = src.e(0), ey = src.e(1), ez = src.e(2);
    const bool xin = i < a.Nx - 1;
    const unsigned PY = a.psi_py, PZ = a.psi_pz, PX = a.psi_px;
    const bool ux = sc.jn && sc.kn, uy = want_y && xin && sc.kn, uz = want_z && xin && sc.jn;
    const unsigned oy = sc.oyh + (unsigned)i * PY, oz = sc.ozh + (unsigned)i * PZ,
                   ox = (unsigned)max(sxh, 0) * PX + sc.ox;
    float *const *W = a.Ph[PAR ^ 1];
    const float p0 = ps.p0, p1 = ps.p1, p2 = ps.p2, p3 = ps.p3, p4 = ps.p4, p5 = ps.p5;
    if (ux) {
        const float dEz = src.ej(2) - ez;
        const float dEy = src.ek(1) - ey;
        float h = a.c1h * o.x - (a.chy * dEz - a.chz * dEy);
        if (sc.syh >= 0) {
            const float p = (YZ == 1 ? sc.bhy : T.Bh[sc.syh]) * p0 + (YZ == 1 ? sc.ahy : T.Ahy[sc.syh]) * dEz;
            if (store_psi) W[0][oy] = p;
            h -= a.c2h * p;
            if (a.kappa_on) h -= a.c2h * ((YZ == 1 ? sc.khy : T.Khy[sc.syh]) * dEz);
        }
        if (sc.szh >= 0) {
            const float p = (YZ == 2 ? sc.bhz : T.Bh[sc.szh]) * p1 + (YZ == 2 ? sc.ahz : T.Ahz[sc.szh]) * dEy;
            if (store_psi) W[1][oz] = p;
            h += a.c2h * p;
            if (a.kappa_on) h += a.c2h * ((YZ == 2 ? sc.khz : T.Khz[sc.szh]) * dEy);
        }
        o.x = h;
    }
    if (uy) {
        const float dEx = src.ek(0) - ex;
        const float dEz = src.ei(2) - ez;
        float h = a.c1h * o.y - (a.chz * dEx - a.chx * dEz);
        if (sxh >= 0) {
            const float p = T.Bh[sxh] * p2 + T.Ahx[sxh] * dEz;
            if (store_psi) W[2][ox] = p;
            h += a.c2h * p;
            if (a.kappa_on) h += a.c2h * (T.Khx[sxh] * dEz);
        }
        if (sc.szh >= 0) {
            const float p = (YZ == 2 ? sc.bhz : T.Bh[sc.szh]) * p3 + (YZ == 2 ? sc.ahz : T.Ahz[sc.szh]) * dEx;
            if (store_psi) W[3][oz] = p;
            h -= a.c2h * p;
            if (a.kappa_on) h -= a.c2h * ((YZ == 2 ? sc.khz : T.Khz[sc.szh]) * dEx);
        }
        o.y = h;
    }
    if (uz) {
        const float dEy = src.ei(1) - ey;
        const float dEx = src.ej(0) - ex;
        float h = a.c1h * o.z - (a.chx * dEy - a.chy * dEx);
        if (sxh >= 0) {
            const float p = T.Bh[sxh] * p4 + T.Ahx[sxh] * dEy;
            if (store_psi) W[4][ox] = p;
            h -= a.c2h * p;
            if (a.kappa_on) h -= a.c2h * (T.Khx[sxh] * dEy);
        }
        if (sc.syh >= 0) {
            const float p = (YZ == 1 ? sc.bhy : T.Bh[sc.syh]) * p5 + (YZ == 1 ? sc.ahy : T.Ahy[sc.syh]) * dEx;
            if (store_psi) W[5][oy] = p;
            h += a.c2h * p;
            if (a.kappa_on) h += a.c2h * ((YZ == 1 ? sc.khy : T.Khy[sc.syh]) * dEx);
        }
        o.z = h;
    }
    return o;
}

template <int PAR, int YZ, class HS>
__device__ __forceinline__ EVal e_slab(const Args &a, const Tables &T, int i, int sxe, float ex, float ey, float ez,
                                       const HVal &hv, const HS &hs, float jx, float jy, float jz,
                                       const SlabCell &sc, const Psi6 &ps) {
    const float c1 = a.c1e0, c2 = a.c2e0, cx = a.cex, cy = a.cey, cz = a.cez;
    const bool iy = i >= 1 && i < a.Nx - 1;
    const bool ux = i < a.Nx - 1 && sc.j1 && sc.jn && sc.k1 && sc.kn, uy = iy && sc.k1, uz = iy && sc.j1;
    const unsigned PY = a.psi_py, PZ = a.psi_pz, PX = a.psi_px;
    const unsigned oy = sc.oye + (unsigned)i * PY, oz = sc.oze + (unsigned)i * PZ,
                   ox = (unsigned)max(sxe, 0) * PX + sc.ox;
    float *const *Pe = a.Pe;
    const float p0 = ps.p0, p1 = ps.p1, p2 = ps.p2, p3 = ps.p3, p4 = ps.p4, p5 = ps.p5;
    if (ux) {
        const float dHz = hv.z - hs.hj(2);
        const float dHy = hv.y - hs.hk(1);
        float e = c1 * ex + (cy * dHz - cz * dHy) - c2 * jx;
        if (sc.sye >= 0) {
            const float p = (YZ == 1 ? sc.bey : T.Be[sc.sye]) * p0 + (YZ == 1 ? sc.aey : T.Aey[sc.sye]) * dHz;
            Pe[0][oy] = p;
            e += a.c2e0 * p;
            if (a.kappa_on) e += a.c2e0 * ((YZ == 1 ? sc.key : T.Key[sc.sye]) * dHz);
        }
        if (sc.sze >= 0) {
            const float p = (YZ == 2 ? sc.bez : T.Be[sc.sze]) * p1 + (YZ == 2 ? sc.aez : T.Aez[sc.sze]) * dHy;
            Pe[1][oz] = p;
            e -= a.c2e0 * p;
            if (a.kappa_on) e -= a.c2e0 * ((YZ == 2 ? sc.kez : T.Kez[sc.sze]) * dHy);
        }
        ex = e;
    }
    if (uy) {
        const float dHx = hv.x - hs.hk(0);
        const float dHz = hv.z - hs.hzi();
        float e = c1 * ey + (cz * dHx - cx * dHz) - c2 * jy;
        if (sxe >= 0) {
            float p = 0.f;
            if (sc.jn && sc.kn) {
                p = T.Be[sxe] * p2 + T.Aex[sxe] * dHz;
                Pe[2][ox] = p;
            }
            e -= a.c2e0 * p;
            if (a.kappa_on) e -= a.c2e0 * (T.Kex[sxe] * dHz);
        }
        if (sc.sze >= 0) {
            float p = 0.f;
            if (sc.jn) {
                p = (YZ == 2 ? sc.bez : T.Be[sc.sze]) * p3 + (YZ == 2 ? sc.aez : T.Aez[sc.sze]) * dHx;
                Pe[3][oz] = p;
            }
            e += a.c2e0 * p;
            if (a.kappa_on) e += a.c2e0 * ((YZ == 2 ? sc.kez : T.Kez[sc.sze]) * dHx);
        }
        ey = e;
    }
    if (uz) {
        const float dHy = hv.y - hs.hyi();
        const float dHx = hv.x - hs.hj(0);
        float e = c1 * ez + (cx * dHy - cy * dHx) - c2 * jz;
        if (sxe >= 0) {
            float p = 0.f;
            if (sc.jn && sc.kn) {
                p = T.Be[sxe] * p4 + T.Aex[sxe] * dHy;
                Pe[4][ox] = p;
            }
            e += a.c2e0 * p;
            if (a.kappa_on) e += a.c2e0 * (T.Kex[sxe] * dHy);
        }
        if (sc.sye >= 0 && sc.kn) {
            const float p = (YZ == 1 ? sc.bey : T.Be[sc.sye]) * p5 + (YZ == 1 ? sc.aey : T.Aey[sc.sye]) * dHx;
            Pe[5][oy] = p;
            e -= a.c2e0 * p;
            if (a.kappa_on) e -= a.c2e0 * ((YZ == 1 ? sc.key : T.Key[sc.sye]) * dHx);
        }
        ez = e;
    }
    return EVal{ex, ey, ez, ez};
}

// The whole 1-D incident line for this step, written to set PAR^1 (one CTA).
template <int PAR>
__device__ void line_update(const Args &a, int t) {
    const int Nx = a.Nx, L = a.L;
    if (a.oblique) {  // auxiliary line along k: E in slot 1, H in slot 2, CPML at the far end
        const int M = a.M;
        const float *e = a.inc[PAR][1], *h = a.inc[PAR][2];
        float *e2 = a.inc[PAR ^ 1][1], *h2 = a.inc[PAR ^ 1][2];
        for (int n = threadIdx.x; n < M; n += blockDim.x) {
            float v = h[n];
            if (n < M - 1) {
                v = a.c1h * h[n] - a.chl * (e[n + 1] - e[n]);
                if (n >= M - L - 1) {
                    const int s = n - a.ashift;
                    const float p = a.tb->Bh1[s] * a.incP[PAR][2][s] + a.tb->Ah1[s] * (e[n + 1] - e[n]);
                    a.incP[PAR ^ 1][2][s] = p;
                    v -= a.c2h * p;
                }
            }
            h2[n] = v;
        }
        __syncthreads();
        for (int n = threadIdx.x; n < M; n += blockDim.x) {
            float v = e[n];
            if (n >= 1 && n < M - 1) {
                v = a.c1e0 * e[n] - a.cel * (h2[n] - h2[n - 1]);
                if (n >= M - L - 1) {
                    const int s = n - a.ashift;
                    const float p = a.tb->Be1[s] * a.incP[PAR][1][s] + a.tb->Ae1[s] * (h2[n] - h2[n - 1]);
                    a.incP[PAR ^ 1][1][s] = p;
                    v -= a.c2e0 * p;
                }
            } else if (n == 0) {
                v = a.src[2 * t];
            }
            e2[n] = v;
        }
        return;
    }
    const float *ey = a.inc[PAR][0], *ez = a.inc[PAR][1], *hy = a.inc[PAR][2], *hz = a.inc[PAR][3];
    float *ey2 = a.inc[PAR ^ 1][0], *ez2 = a.inc[PAR ^ 1][1], *hy2 = a.inc[PAR ^ 1][2],
          *hz2 = a.inc[PAR ^ 1][3];
    for (int i = threadIdx.x; i < Nx; i += blockDim.x) {
        float vy = hy[i], vz = hz[i];
        if (i < Nx - 1) {
            vy = a.c1h * hy[i] + a.chx * (ez[i + 1] - ez[i]);
            vz = a.c1h * hz[i] - a.chx * (ey[i + 1] - ey[i]);
            if (a.dopml && i >= Nx - L - 1) {
                const int s = i - a.xshift;
                const float py = a.tb->Bh[s] * a.incP[PAR][2][s] + a.tb->Ahx[s] * (ez[i + 1] - ez[i]);
                const float pz = a.tb->Bh[s] * a.incP[PAR][3][s] + a.tb->Ahx[s] * (ey[i + 1] - ey[i]);
                a.incP[PAR ^ 1][2][s] = py;
                a.incP[PAR ^ 1][3][s] = pz;
                vy += a.c2h * py;
                vz -= a.c2h * pz;
            }
        }
        hy2[i] = vy;
        hz2[i] = vz;
    }
    __syncthreads();
    for (int i = threadIdx.x; i < Nx; i += blockDim.x) {
        float vy = ey[i], vz = ez[i];
        if (i >= 1 && i < Nx - 1) {
            vy = a.c1e0 * ey[i] - a.cex * (hz2[i] - hz2[i - 1]);
            vz = a.c1e0 * ez[i] + a.cex * (hy2[i] - hy2[i - 1]);
            if (a.dopml && i >= Nx - L - 1) {
                const int s = i - a.xshift;
                const float py = a.tb->Be[s] * a.incP[PAR][0][s] + a.tb->Aex[s] * (hz2[i] - hz2[i - 1]);
                const float pz = a.tb->Be[s] * a.incP[PAR][1][s] + a.tb->Aex[s] * (hy2[i] - hy2[i - 1]);
                a.incP[PAR ^ 1][0][s] = py;
                a.incP[PAR ^ 1][1][s] = pz;
                vy -= a.c2e0 * py;
                vz += a.c2e0 * pz;
            }
        } else if (i == 0) {
            vz = a.src[2 * t];
            vy = a.src[2 * t + 1];
        }
        ey2[i] = vy;
        ez2[i] = vz;
    }
}

// Everything a marching CTA keeps between planes.
struct MarchCtx {
    unsigned char *smem;
    float *hn;
    uint64_t *bar;
    int tid, warp, lane, j0, k0, i_begin, i_end, p0, q_last, dj, dk, j, k;
    bool role_ok, in_grid, valid;
    int issued;
    int tile_id;
    const Tables *tbs;  // MARCH_SLAB: the CPML tables, copied to shared memory
};

// Shared-memory layout after the stages and new-H planes: NS stage barriers,
// three poll flags (16 bytes), then the plasma flags of planes p0, p0+1, ...
__device__ __forceinline__ unsigned char *pflags(const MarchCtx &c) {
    return (unsigned char *)(c.bar + NS) + 16;
}

// Does the tile's block of plane q hold plasma?  (See Args::plasma.)  The
// flags of the CTA's first PF_CAP planes are copied to shared memory when the
// item starts: read from global memory, the flag's latency (about 500 cycles
// from L2) sat at the start of every plane.
__device__ __forceinline__ bool plasma_at(const Args &a, const MarchCtx &c, int q) {
    if (!a.plasma) return true;
    const int r = q - c.p0;
    return r < PF_CAP ? pflags(c)[r] != 0 : a.plasma[(size_t)q * a.ntiles + c.tile_id] != 0;
}

// Stage of plane q: the six field boxes, one copy.  (J is read from global
// memory, and only in blocks holding plasma: keeping it out of the stages
// leaves 15 KB of each CTA's shared memory to L1, which measured faster than
// staging it.)
template <int PAR>
__device__ __forceinline__ void issue_stage(const Maps &maps, MarchCtx &c, int q) {
    const int slot = (q - c.p0) % NS;
    unsigned char *dst = c.smem + slot * STAGE_B;
    mbar_arm(&c.bar[slot], STAGE_TX);
    tma4(dst, &maps.F[PAR], c.k0 - 4, c.j0 - 1, q, 0, &c.bar[slot]);
}

// Lagged current update of one cell (source/meteor-fork.cpp:1539-1595), the
// form the fast pass and the band kernels share: J of step t-1 advanced from
// the E at the start of pass t (exo, eyo, ezo; exim, eyjm, ezkm are Ex at
// i-1, Ey at j-1, Ez at k-1, used by the node-averaged Lee-Kalluri update).
// `m`: the 18 Lee-Kalluri coefficients (JM 1, 2).
template <int JM>
__device__ __forceinline__ void j_advance(const Args &a, const float *m, float cwq, float cnu, float Gk, float G2k,
                                          float exo, float eyo, float ezo, float exim, float eyjm, float ezkm,
                                          float &jx, float &jy, float &jz) {
    const float wq = cwq * G2k;
    if (JM == 0) {
        const float nue = cnu * Gk;
        const float den = 2.f + nue * a.dtf;
        const float ca = (2.f - nue * a.dtf) / den;
        const float cb = (2.f * a.dtf) * wq / den;
        jx = ca * jx + cb * exo;
        jy = ca * jy + cb * eyo;
        jz = ca * jz + cb * ezo;
    } else {
        const bool co = a.lk_colocated;
        const float m0 = co ? exo : 0.5f * (exo + exim);
        const float m1 = co ? eyo : 0.5f * (eyo + eyjm);
        const float m2 = co ? ezo : 0.5f * (ezo + ezkm);
        const float nx = m[0] * jx + m[1] * jy + m[2] * jz + wq * (m[9] * m0 + m[10] * m1 + m[11] * m2);
        const float ny = m[3] * jx + m[4] * jy + m[5] * jz + wq * (m[12] * m0 + m[13] * m1 + m[14] * m2);
        const float nz = m[6] * jx + m[7] * jy + m[8] * jz + wq * (m[15] * m0 + m[16] * m1 + m[17] * m2);
        jx = nx; jy = ny; jz = nz;
    }
}

// How a CTA marches its planes (template parameter of march and run_item):
//   MARCH_GENERAL: per tile and plane, the fast path where it applies, else
//     the general path (CPML, domain edges, TF/SF, slices as Args says);
//   MARCH_FAST: a clean tile whose every plane is an interior one (oblique
//     TF/SF corrections after the pass, no record step, the CPML slabs and
//     domain edges left to other work): the warm-up plane also takes the fast
//     path (its H only), and the general path is not compiled in;
//   MARCH_SLAB: the CPML slabs and domain edges (k_fp32_slab): every cell
//     takes the CPML path of h_slab / e_slab.
enum : int { MARCH_GENERAL = 0, MARCH_FAST = 1, MARCH_SLAB = 2 };

// The plane loop of one CTA.  Returns the plane at which a TMA wait ran out,
// or -1.
template <int PAR, int JM, bool CLEAN, int MODE = MARCH_GENERAL, bool PSIPF = true, int YZ = 3>
__device__ __forceinline__ int march(const Maps &maps, const Args &a, MarchCtx &c, int t, int record,
                                     bool tf_in) {
    constexpr bool FASTONLY = MODE == MARCH_FAST, SLAB = MODE == MARCH_SLAB;
    // per-item CPML coefficients (slab_coef) where the registers allow: not in
    // the three-CTAs-per-SM form without the psi prefetch
    constexpr int CYZ = PSIPF ? YZ : 3;
    const int Nx = a.Nx, Ny = a.Ny, Nz = a.Nz, L = a.L;
    const size_t plane = (size_t)Ny * a.Nzp;
    const int dj = c.dj, dk = c.dk, j = c.j, k = c.k, warp = c.warp;
    const bool tile = warp < TJ;
    const bool valid = c.valid, in_grid = c.in_grid;

    // J method: JM 0 = Young DI, 1 = Lee-Kalluri with one matrix pair for the
    // whole grid (read from the constant bank), 2 = Lee-Kalluri table.
    float lkm[JM == 2 ? 18 : 1];
    if (JM == 2 && a.lk_mode == LK_PER_K && valid)
        for (int q = 0; q < 18; q++) lkm[q] = a.lk[(size_t)k * 18 + q];
    const float Gk = valid ? a.G[k] : 0.f, G2k = valid ? a.G2[k] : 0.f;
    const size_t col = (size_t)(valid ? j : 0) * a.Nzp + (valid ? k : 0);

    // The plasma weight (and collision frequency) of the thread's cell is
    // prefetched one plane ahead into registers, so its latency overlaps the
    // previous plane's work.  (In the general path, prefetching the x-normal
    // CPML psi the same way was measured slower: the registers it holds
    // across the plane loop made the boundary path spill.  The slab march,
    // at two CTAs per SM, prefetches all of its cell's psi values: Psi6.)
    const int jj = valid ? j : 0, kk = valid ? k : 0;
    auto pf_load = [&](int qq, float &wq, float &nu) {
        if (!valid || qq >= Nx) return;
        const size_t ij = (size_t)qq * Ny + jj;
        const size_t cq = (size_t)qq * plane + (size_t)jj * a.Nzp + kk;
        wq = a.wq3 ? a.wq3[cq] : a.wq2[ij];
        if (JM == 0) nu = a.nu3 ? a.nu3[cq] : a.nu2[ij];

    };
    float nwq = 0.f, nnu = 0.f;
    bool npl = plasma_at(a, c, c.p0);
    if (npl) pf_load(c.p0, nwq, nnu);

    // One thread polls the stage mbarriers; the rest of the CTA sleeps in the
    // CTA barrier instead of spinning.  The poller's mbarrier acquire plus
    // bar.sync make the TMA data visible to every thread.
    // One CTA barrier per x plane, between the H and the E updates:
    //   * before it the poller waits for the stage plane q+1's H will read
    //     (plane q+2's E box);
    //   * after it every thread has finished plane q-1 (its E update came
    //     before plane q's H), so the producer refills plane q-1's slot with
    //     plane q-1+NS, and the new-H plane alternates between two buffers so
    //     plane q+1's H never overwrites values plane q's E still reads;
    //   * the poll flag alternates as well, so a fast thread never overwrites
    //     the flag a slow thread has not read yet.
    volatile int *okflag = (volatile int *)(c.bar + NS);
    auto stage_ready = [&](int qq) {
        return qq > c.q_last || mbar_wait(&c.bar[(qq - c.p0) % NS], ((qq - c.p0) / NS) & 1);
    };
    if (c.tid == PROD) okflag[2] = (stage_ready(c.p0) && stage_ready(c.p0 + 1)) ? 1 : 0;
    __syncthreads();
    if (!okflag[2]) return c.p0;
    auto mid_plane = [&](int q) -> bool {
        if (c.tid == PROD) okflag[q & 1] = stage_ready(q + 2) ? 1 : 0;
        __syncthreads();
        if (!okflag[q & 1]) return false;
        if (c.tid == PROD && q > c.p0 && q - 1 + NS <= c.q_last) {
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            issue_stage<PAR>(maps, c, q - 1 + NS);
            c.issued = q - 1 + NS;
        }
        return true;
    };

    float hy_prev = 0.f, hz_prev = 0.f, ex_prev = 0.f;
    SlabCell sc{};
    Psi6 nhp{0.f, 0.f, 0.f, 0.f, 0.f, 0.f}, nep = nhp;  // SLAB with PSIPF: psi of the next plane
    // SLAB: the next plane's x-slab indices (plane-uniform), computed once
    // for the prefetch and the update
    int nsxh = hslab(c.p0, Nx, L, a.xshift), nsxe = eslab(c.p0, Nx, L, a.xshift);
    if constexpr (SLAB) {
        sc = slab_coef<CYZ>(slab_view<YZ>(slab_cell(a, j, k)), *c.tbs);
        if (PSIPF && in_grid) {
            nhp = h_slab_psi<PAR>(a, c.p0, nsxh, sc, warp != TJ, warp != TJ + 1);
            if (valid && c.p0 >= c.i_begin) nep = e_slab_psi(a, c.p0, nsxe, sc);
        }
    }
    // The stage slot of plane q and the cell offset advance with q (no
    // modulo or 64-bit multiply per plane).
    int slot = 0;
    size_t cg = (size_t)c.p0 * plane + col;
    for (int q = c.p0; q < c.i_end; q++, cg += plane) {
        const int i = q;
        const float cwq = nwq, cnu = nnu;
        const bool pl = npl;  // this plane's block holds plasma
        npl = q + 1 < c.i_end && plasma_at(a, c, q + 1);
        if (npl) pf_load(q + 1, nwq, nnu);
        Psi6 hps{0.f, 0.f, 0.f, 0.f, 0.f, 0.f}, eps = hps;  // SLAB: this plane's psi
        const int sxh = nsxh, sxe = nsxe;
        if constexpr (SLAB) {
            nsxh = hslab(q + 1, Nx, L, a.xshift);
            nsxe = eslab(q + 1, Nx, L, a.xshift);
        }
        if constexpr (SLAB && PSIPF) {
            hps = nhp;
            eps = nep;
            if (in_grid && q + 1 < c.i_end) {
                nhp = h_slab_psi<PAR>(a, q + 1, nsxh, sc, warp != TJ, warp != TJ + 1);
                if (valid && q + 1 >= c.i_begin) nep = e_slab_psi(a, q + 1, nsxe, sc);
            }
        }
        const int slot1 = slot == NS - 1 ? 0 : slot + 1;
        float *hn = c.hn + (q & 1) * (align128(HN_B) / 4);  // this plane's new-H buffer
        // Stages q and q+1 are resident: the barrier of the previous plane
        // (or the one before the loop) guarantees it.
        const Stage s = stage_at(c.smem + slot * STAGE_B);
        const Stage s1 = stage_at(c.smem + slot1 * STAGE_B);
        slot = slot1;
        const bool real = q >= c.i_begin;

        // Interior fast path: a clean tile on a plane outside the x CPML slabs
        // and away from every x-special plane (TF/SF faces when the tile is in
        // the box and the corrections are made here, the x slice on record
        // steps).  No conditionals per cell; the arithmetic is the same as the
        // general path's.
        const int xlo = a.band ? 0 : a.dopml ? L + 1 : 1, xhi = a.band ? Nx - 1 : a.dopml ? Nx - L - 2 : Nx - 2;
        const bool x_tfsf = (!a.oblique || a.obl_inline) && tf_in &&
                            (i == a.bx1 - 1 || i == a.bx1 || i == a.bx2 - 1);
        const bool fast = FASTONLY || (!SLAB && CLEAN && real && i >= xlo && i <= xhi &&
                                        !(record && i == a.ssx) && !x_tfsf);
        if (fast) {
            // With the band kernels a clean tile may reach past the grid
            // (`valid` false) or hold domain-edge cells, where J is not
            // advanced (their E and H are recomputed by the band kernels).
            float jx = 0.f, jy = 0.f, jz = 0.f, exo = 0.f, eyo = 0.f, ezo = 0.f;
            if (c.role_ok) {  // the cell's old E, for J, H and E
                exo = s.e[0][EIDX(dj, dk)];
                eyo = s.e[1][EIDX(dj, dk)];
                ezo = s.e[2][EIDX(dj, dk)];
            }
            if (valid && real && pl) {
                jx = a.J[0][cg];
                jy = a.J[1][cg];
                jz = a.J[2][cg];
                if (t > 0 && (!a.band || (i >= 1 && i < Nx - 1 && j >= 1 && j < Ny - 1 && k >= 1 && k < Nz - 1))) {
                    const float *m = JM == 1 ? a.lku : lkm;
                    float tbl[JM == 2 ? 18 : 1];
                    if (JM == 2 && a.lk_mode != LK_PER_K) {
                        const size_t e = a.lk_mode == LK_PER_IJ ? (size_t)i * Ny + j : cg;
                        for (int u = 0; u < 18; u++) tbl[u] = a.lk[e * 18 + u];
                        m = tbl;
                    }
                    j_advance<JM>(a, m, cwq, cnu, Gk, G2k, exo, eyo, ezo, ex_prev, s.e[1][EIDX(dj - 1, dk)],
                                  s.e[2][EIDX(dj, dk - 1)], jx, jy, jz);
                }
            }
            HVal hv = {0.f, 0.f, 0.f};
            if (c.role_ok) {
                const float ex = exo, ey = eyo, ez = ezo;
                hv.x = a.c1h * s.h[0][HIDX(dj, dk)] -
                       (a.chy * (s.e[2][EIDX(dj + 1, dk)] - ez) - a.chz * (s.e[1][EIDX(dj, dk + 1)] - ey));
                HN(0, dj, dk) = hv.x;
                if (warp != TJ) {
                    hv.y = a.c1h * s.h[1][HIDX(dj, dk)] -
                           (a.chz * (s.e[0][EIDX(dj, dk + 1)] - ex) - a.chx * (s1.e[2][EIDX(dj, dk)] - ez));
                    HN(1, dj, dk) = hv.y;
                }
                if (warp != TJ + 1) {
                    hv.z = a.c1h * s.h[2][HIDX(dj, dk)] -
                           (a.chx * (s1.e[1][EIDX(dj, dk)] - ey) - a.chy * (s.e[0][EIDX(dj + 1, dk)] - ex));
                    HN(2, dj, dk) = hv.z;
                }
            }
            if (valid && real) {
                a.H[PAR ^ 1][0][cg] = hv.x;
                a.H[PAR ^ 1][1][cg] = hv.y;
                a.H[PAR ^ 1][2][cg] = hv.z;
            }
            if (!mid_plane(q)) return q + 2;
            if (valid) {
                if (real) {
                    const float c1 = a.c1e0, c2 = a.c2e0;
                    const float ex = c1 * exo + (a.cey * (hv.z - HN(2, dj - 1, dk)) - a.cez * (hv.y - HN(1, dj, dk - 1))) - c2 * jx;
                    const float ey = c1 * eyo + (a.cez * (hv.x - HN(0, dj, dk - 1)) - a.cex * (hv.z - hz_prev)) - c2 * jy;
                    const float ez = c1 * ezo + (a.cex * (hv.y - hy_prev) - a.cey * (hv.x - HN(0, dj - 1, dk))) - c2 * jz;
                    a.E[PAR ^ 1][0][cg] = ex;
                    a.E[PAR ^ 1][1][cg] = ey;
                    a.E[PAR ^ 1][2][cg] = ez;
                    if (pl) {
                        a.J[0][cg] = jx;
                        a.J[1][cg] = jy;
                        a.J[2][cg] = jz;
                    }
                }
                ex_prev = exo;
            }
            hy_prev = hv.y;
            hz_prev = hv.z;
            continue;
        }

        // ---- J of the previous step (lagged), source/meteor-fork.cpp:1523-1595
        float jx = 0.f, jy = 0.f, jz = 0.f;
        if (valid && real && pl) {
            jx = a.J[0][cg];
            jy = a.J[1][cg];
            jz = a.J[2][cg];
            const bool jdom = (CLEAN && !a.band && !SLAB)
                                  ? (i >= 1 && i < Nx - 1)
                                  : (i >= 1 && i < Nx - 1 && j >= 1 && j < Ny - 1 && k >= 1 && k < Nz - 1);
            if (t > 0 && jdom) {
                const float exc = s.e[0][EIDX(dj, dk)], eyc = s.e[1][EIDX(dj, dk)],
                            ezc = s.e[2][EIDX(dj, dk)];
                const size_t ij = (size_t)i * Ny + j;
                const float wq = cwq * G2k;
                if (JM == 0) {
                    const float nue = cnu * Gk;
                    const float den = 2.f + nue * a.dtf;
                    const float ca = (2.f - nue * a.dtf) / den;
                    const float cb = (2.f * a.dtf) * wq / den;
                    jx = ca * jx + cb * exc;
                    jy = ca * jy + cb * eyc;
                    jz = ca * jz + cb * ezc;
                } else {
                    const bool co = a.lk_colocated;
                    const float m0 = co ? exc : 0.5f * (exc + ex_prev);
                    const float m1 = co ? eyc : 0.5f * (eyc + s.e[1][EIDX(dj - 1, dk)]);
                    const float m2 = co ? ezc : 0.5f * (ezc + s.e[2][EIDX(dj, dk - 1)]);
                    const float *m = JM == 1 ? a.lku : lkm;
                    float tbl[JM == 2 ? 18 : 1];
                    if (JM == 2 && a.lk_mode != LK_PER_K) {
                        const size_t e = a.lk_mode == LK_PER_IJ ? ij : cg;
                        for (int u = 0; u < 18; u++) tbl[u] = a.lk[e * 18 + u];
                        m = tbl;
                    }
                    const float nx = m[0] * jx + m[1] * jy + m[2] * jz + wq * (m[9] * m0 + m[10] * m1 + m[11] * m2);
                    const float ny = m[3] * jx + m[4] * jy + m[5] * jz + wq * (m[12] * m0 + m[13] * m1 + m[14] * m2);
                    const float nz = m[6] * jx + m[7] * jy + m[8] * jz + wq * (m[15] * m0 + m[16] * m1 + m[17] * m2);
                    jx = nx; jy = ny; jz = nz;
                }
            }
        }

        // ---- H of this plane: tile (all comps), halo row (Hx, Hz), halo column (Hx, Hy)
        HVal hv = {0.f, 0.f, 0.f};
        if constexpr (SLAB) {
            if (in_grid) {
                if constexpr (!PSIPF) hps = h_slab_psi<PAR>(a, i, sxh, sc, warp != TJ, warp != TJ + 1);
                hv = h_slab<PAR, CYZ>(a, *c.tbs, i, sxh, StageSrc{s, s1, dj, dk}, sc, tile && real,
                                 warp != TJ, warp != TJ + 1, hps);
            }
        } else {
            if (in_grid)
                hv = h_cell<PAR, CLEAN>(a, i, j, k, StageSrc{s, s1, dj, dk}, tile && real, warp != TJ,
                                        warp != TJ + 1, tf_in, a.dopml && !a.band);
        }
        if (c.role_ok) {
            HN(0, dj, dk) = hv.x;
            if (warp != TJ) HN(1, dj, dk) = hv.y;
            if (warp != TJ + 1) HN(2, dj, dk) = hv.z;
        }
        if (valid && real) {
            a.H[PAR ^ 1][0][cg] = hv.x;
            a.H[PAR ^ 1][1][cg] = hv.y;
            a.H[PAR ^ 1][2][cg] = hv.z;
        }
        if (!mid_plane(q)) return q + 2;

        // ---- E of this plane (tile), source/meteor-2.1.cpp:1020-1374
        if (valid && real) {
            const float ex_old = s.e[0][EIDX(dj, dk)];
            EVal ev;
            if constexpr (SLAB && !PSIPF) eps = e_slab_psi(a, i, sxe, sc);
            if constexpr (SLAB)
                ev = e_slab<PAR, CYZ>(a, *c.tbs, i, sxe, ex_old, s.e[1][EIDX(dj, dk)],
                                 s.e[2][EIDX(dj, dk)], hv, StageHSrc{hn, dj, dk, hy_prev, hz_prev}, jx, jy, jz, sc,
                                 eps);
            else
                ev = e_cell<PAR, CLEAN>(a, i, j, k, ex_old, s.e[1][EIDX(dj, dk)], s.e[2][EIDX(dj, dk)], hv,
                                        StageHSrc{hn, dj, dk, hy_prev, hz_prev}, jx, jy, jz, tf_in,
                                        a.dopml && !a.band);
            const float ex = ev.x, ey = ev.y, ez = ev.z, ez_slice = ev.z_slice;
            a.E[PAR ^ 1][0][cg] = ex;
            a.E[PAR ^ 1][1][cg] = ey;
            a.E[PAR ^ 1][2][cg] = ez;
            if (pl) {
                a.J[0][cg] = jx;
                a.J[1][cg] = jy;
                a.J[2][cg] = jz;
            }

            // ---- slices on record steps
            if (!SLAB && record) {
                const size_t oz = 0, oy = 2 * (size_t)Nx * Ny, ox = oy + 2 * (size_t)Nx * Nz;
                if (!CLEAN && k == a.ssz) {
                    a.slE[oz + (size_t)i * Ny + j] = ey;
                    a.slE[oz + (size_t)Nx * Ny + (size_t)i * Ny + j] = ez_slice;
                    if (j < Ny - 1) {
                        a.slH[oz + (size_t)i * Ny + j] = hv.y;
                        a.slH[oz + (size_t)Nx * Ny + (size_t)i * Ny + j] = hv.z;
                    }
                }
                if (!CLEAN && j == a.ssy) {
                    a.slE[oy + (size_t)i * Nz + k] = ey;
                    a.slE[oy + (size_t)Nx * Nz + (size_t)i * Nz + k] = ez_slice;
                    if (k < Nz - 1) {
                        a.slH[oy + (size_t)i * Nz + k] = hv.y;
                        a.slH[oy + (size_t)Nx * Nz + (size_t)i * Nz + k] = hv.z;
                    }
                }
                if (i == a.ssx) {
                    a.slE[ox + (size_t)j * Nz + k] = ey;
                    a.slE[ox + (size_t)Ny * Nz + (size_t)j * Nz + k] = ez_slice;
                    if ((CLEAN && !a.band) || (j < Ny - 1 && k < Nz - 1)) {
                        a.slH[ox + (size_t)j * Nz + k] = hv.y;
                        a.slH[ox + (size_t)Ny * Nz + (size_t)j * Nz + k] = hv.z;
                    }
                }
            }
            ex_prev = ex_old;
        } else if (valid) {
            ex_prev = s.e[0][EIDX(dj, dk)];  // warm-up plane
        }
        hy_prev = hv.y;
        hz_prev = hv.z;
    }
    return -1;
}

// Probes of the previous step from the read set (source/meteor-2.1.cpp:1443-1455),
// by lanes 8.. of warp 9 of the item that advances the incident line.
template <int PAR>
__device__ __forceinline__ void record_probes(const Args &a, int t) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (warp != 9 || lane < 8 || lane - 8 >= a.nprobes) return;
    const int pidx = lane - 8;
    const int ix = a.probe_ijk[3 * pidx], iy = a.probe_ijk[3 * pidx + 1], iz = a.probe_ijk[3 * pidx + 2];
    const size_t sI = (size_t)a.Ny * a.Nzp, sJ = a.Nzp;
    const size_t cc = ix * sI + iy * sJ + iz;
    const float *E0 = a.E[PAR][0], *E1 = a.E[PAR][1], *E2 = a.E[PAR][2];
    const float *H0 = a.H[PAR][0], *H1 = a.H[PAR][1], *H2 = a.H[PAR][2];
    const size_t o = (size_t)(t - 1) * a.nprobes + pidx, T = (size_t)a.tsteps * a.nprobes;
    a.probe[o] = 0.5 * ((double)E0[cc] + E0[cc - sI]);
    a.probe[T + o] = 0.5 * ((double)E1[cc] + E1[cc - sJ]);
    a.probe[2 * T + o] = 0.5 * ((double)E2[cc] + E2[cc - 1]);
    a.probe[3 * T + o] = 0.25 * ((double)H0[cc] + H0[cc - sJ] + H0[cc - 1] + H0[cc - sJ - 1]);
    a.probe[4 * T + o] = 0.25 * ((double)H1[cc] + H1[cc - sI] + H1[cc - 1] + H1[cc - sI - 1]);
    a.probe[5 * T + o] = 0.25 * ((double)H2[cc] + H2[cc - sJ] + H2[cc - sI] + H2[cc - sI - sJ]);
}

// ---------------------------------------------------------------------------
// One work item: tile `tile_id` of simulation `a` over the planes
// [i_begin, i_end).  The item with `first` set also advances the incident line
// and records the probes of the previous step.  `inited` says whether the
// CTA's stage mbarriers hold an earlier item's objects (they are invalidated
// and re-initialised).  Returns false when a bounded wait ran out (the
// simulation's error flag is then set).
template <int PAR, int JM, int MODE = MARCH_GENERAL, bool PSIPF = true, int YZ = 3>
__device__ __forceinline__ bool run_item(const Maps &maps, const Args &a, int tile_id, int i_begin, int i_end,
                                         bool first, int t, int record, unsigned char *smem_raw,
                                         bool inited) {
    MarchCtx c;
    // TMA destinations must be 128-byte aligned; the launch reserves 128 spare bytes.
    c.smem = smem_raw + ((128u - (smem_u32(smem_raw) & 127u)) & 127u);
    c.hn = (float *)(c.smem + NS * STAGE_B);
    c.bar = (uint64_t *)(c.smem + NS * STAGE_B + 2 * align128(HN_B));

    c.tid = threadIdx.x;
    c.warp = c.tid >> 5;
    c.lane = c.tid & 31;
    const int Nx = a.Nx, Ny = a.Ny, Nz = a.Nz;
    c.tile_id = tile_id;
    c.k0 = (tile_id % a.ntk) * TK;
    c.j0 = (tile_id / a.ntk) * TJ;
    c.i_begin = i_begin;
    c.i_end = i_end;
    if (c.i_begin >= c.i_end) return true;
    c.p0 = max(c.i_begin - 1, 0);
    c.q_last = min(c.i_end, Nx - 1);  // last plane loaded

    if (first) line_update<PAR>(a, t);

    if (first && t > 0) record_probes<PAR>(a, t);

    if (c.tid == PROD) {
        // An earlier item's barriers have no pending operation (every stage it
        // issued was waited for), so they can be invalidated and reused.
        if (inited)
            for (int s = 0; s < NS; s++)
                asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(smem_u32(&c.bar[s])) : "memory");
        for (int s = 0; s < NS; s++) mbar_init(&c.bar[s], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    // Plasma flags of the item's planes, read through plasma_at after the barrier.
    if (a.plasma && c.tid < PF_CAP && c.tid < c.i_end - c.p0)
        pflags(c)[c.tid] = a.plasma[(size_t)(c.p0 + c.tid) * a.ntiles + tile_id];
    if constexpr (MODE == MARCH_SLAB) {  // the CPML tables, read per cell by the slab march
        float *dst = (float *)(c.smem + SLAB_TB_OFF);
        const float *src = (const float *)a.tb;
        for (int q = c.tid; q < (int)(sizeof(Tables) / 4); q += NTHREADS) dst[q] = src[q];
        c.tbs = (const Tables *)dst;
    }
    __syncthreads();
    c.issued = c.p0 - 1;
    if (c.tid == PROD) {
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        for (int q = c.p0; q <= c.q_last && q < c.p0 + NS; q++) {
            issue_stage<PAR>(maps, c, q);
            c.issued = q;
        }
    }

    // role of this thread
    const bool tile = c.warp < TJ;
    c.dj = tile ? c.warp : (c.warp == TJ ? -1 : c.lane);
    c.dk = tile ? c.lane : (c.warp == TJ ? c.lane : -1);
    c.j = c.j0 + c.dj;
    c.k = c.k0 + c.dk;
    c.role_ok = tile || c.warp == TJ || (c.warp == TJ + 1 && c.lane < TJ);
    c.in_grid = c.role_ok && c.j >= 0 && c.j < Ny && c.k >= 0 && c.k < Nz;
    c.valid = tile && c.in_grid;

    int fail_q;
    if constexpr (MODE == MARCH_SLAB) {
        fail_q = march<PAR, JM, false, MARCH_SLAB, PSIPF, YZ>(maps, a, c, t, 0, false);
    } else {
        const TileInfo ti = classify(a, c.j0, c.k0, record);
        if constexpr (MODE == MARCH_FAST)
            fail_q = march<PAR, JM, true, MARCH_FAST>(maps, a, c, t, 0, ti.tf_in);
        else
            fail_q = ti.clean ? march<PAR, JM, true>(maps, a, c, t, record, ti.tf_in)
                              : march<PAR, JM, false>(maps, a, c, t, record, false);
    }
    if (fail_q >= 0 && c.tid == PROD) {
        atomicOr(a.err, 1u);
        // Let the copies already issued land (bounded) before the CTA exits.
        for (int qq = fail_q; qq <= c.issued; qq++) {
            const int sl = (qq - c.p0) % NS;
            const unsigned pp = ((qq - c.p0) / NS) & 1;
            const uint64_t t0 = globaltimer();
            while (!mbar_test(&c.bar[sl], pp) && globaltimer() - t0 < 200000000ull) {
            }
        }
    }
    return fail_q < 0;
}

// One time step of one simulation: one CTA per (tile, x-chunk).  Boundary
// tiles (general path, several times the work of an interior tile) are
// launched first so that they overlap the bulk of the grid instead of forming
// a tail.  (Running them as a separate launch with a larger register budget on
// a second stream was measured slower: the block scheduler dispatches that
// launch's CTAs ahead of the interior ones, so the two do not overlap.)
template <int PAR, int JM>
__global__ void __launch_bounds__(NTHREADS, JM == 2 ? 2 : 3)
    k_fp32_step(const __grid_constant__ Maps maps, const __grid_constant__ Args a, int t, int record) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    const bool first = blockIdx.x == 0 && blockIdx.y == 0 && blockIdx.z == 0;
    const int ib = a.xbeg + (int)blockIdx.z * a.chunk;
    run_item<PAR, JM>(maps, a, a.tile_order[blockIdx.x], ib, min(a.xend, ib + a.chunk), first, t, record, smem_raw,
                      false);
}

// The same pass when every tile and plane takes the fast path (Args::band,
// oblique TF/SF corrections after the pass, no plate or sphere, no record
// step; see march): without the general path the kernel fits 48 registers,
// four CTAs per SM.
template <int PAR, int JM>
__global__ void __launch_bounds__(NTHREADS, 4)
    k_fp32_step_fast(const __grid_constant__ Maps maps, const __grid_constant__ Args a, int t) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    const bool first = blockIdx.x == 0 && blockIdx.y == 0 && blockIdx.z == 0;
    const int ib = a.xbeg + (int)blockIdx.z * a.chunk;
    run_item<PAR, JM, MARCH_FAST>(maps, a, a.tile_order[blockIdx.x], ib, min(a.xend, ib + a.chunk), first, t, 0,
                                  smem_raw, false);
}

// The CPML slabs and domain edges of a non-record step, as marches of their
// own (MARCH_SLAB), run on a second stream alongside k_fp32_step_wide, which
// marches the tile pairs whose every cell is interior in j and k over every
// plane (the x-slab planes with their x-normal CPML terms).  A work item is
// (tile, first plane, end plane): the tiles that reach into the y or z slabs
// (or past the grid), and interior tiles left without a partner, over all
// planes in x-chunks.  The two kernels write disjoint cells of the new state
// and read the old one, so they need no ordering; each CTA recomputes the
// halo H its E update needs, as in the pass.  The CPML corrections are those
// of the general path (h_cell, e_cell) in lean form (h_slab, e_slab), equal
// to the pass-plus-band-kernels results up to FP32 rounding.  Each thread
// loads its cell's psi values one plane ahead (Psi6), which takes their
// latency off the plane loop; the registers that holds limit the kernel to
// two CTAs per SM (at three it spills and runs slower).
template <int PAR, int JM>
__global__ void __launch_bounds__(NTHREADS, 2)
    k_fp32_slab(const __grid_constant__ Maps maps, const __grid_constant__ Args a, int t,
                const int4 *__restrict__ items) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    const int4 w = items[blockIdx.x];  // (tile, first plane, end plane, YZ: see slab_view)
    if (w.w == 0) run_item<PAR, JM, MARCH_SLAB, true, 0>(maps, a, w.x, w.y, w.z, false, t, 0, smem_raw, false);
    else if (w.w == 1) run_item<PAR, JM, MARCH_SLAB, true, 1>(maps, a, w.x, w.y, w.z, false, t, 0, smem_raw, false);
    else if (w.w == 2) run_item<PAR, JM, MARCH_SLAB, true, 2>(maps, a, w.x, w.y, w.z, false, t, 0, smem_raw, false);
    else run_item<PAR, JM, MARCH_SLAB>(maps, a, w.x, w.y, w.z, false, t, 0, smem_raw, false);
}

// ---------------------------------------------------------------------------
// The interior pass with two cells per thread (k_fp32_step_wide), run with the
// slab march: tiles of TJ x TKW = 8 x 64 (j, k) columns -- two neighbouring
// 8 x 32 tiles -- whose every cell is interior in j and k, over the interior
// planes [w, Nx - w).  Each tile thread owns the cells k0 + 2 lane and
// k0 + 2 lane + 1 of its row: stage reads, new-H plane writes and global
// stores move both cells as one 8-byte access (ld.shared.v2, st.shared.v2,
// st.global.v2: a warp stores 256 contiguous bytes per instruction), and the
// per-plane work that does not depend on the cell (loop, plasma flag, stage
// addresses, the barrier) is shared by the two.  The -k neighbour of the
// second cell is the first cell, in registers.  Warp 8 recomputes H on the
// halo row j0 - 1 (two cells per lane), warp 9 on the halo column k0 - 1
// (lanes 0-7).  The arithmetic is the fast path's, cell by cell.
constexpr int TKW = 2 * TK;                   // tile columns
constexpr int EKW = TKW + 8;                  // box columns k0-4 .. k0+TKW+3
constexpr int C_BW = EJ * EKW * 4;            // one component's box
constexpr int STAGE_BW = align128(6 * C_BW);
constexpr int STAGE_TXW = 6 * C_BW;
constexpr int HNW_COLS = TKW + 2;             // new-H plane columns k0-2 .. k0+TKW-1
constexpr int HNW_B = 3 * HJ * HNW_COLS * 4;
constexpr int SMEM_BW = NS * STAGE_BW + 2 * align128(HNW_B) + NS * 8 + 16 + PF_CAP + 128;
constexpr int SMEM_BATCHW = SMEM_BW > SMEM_BS ? SMEM_BW : SMEM_BS;  // a batch CTA runs either layout
#define EW(dj, dk) (((dj) + 1) * EKW + (dk) + 4)
#define HNW(c, dj, dk) (((c) * HJ + (dj) + 1) * HNW_COLS + (dk) + 2)

__device__ __forceinline__ float2 lds2(const float *p) { return *reinterpret_cast<const float2 *>(p); }
__device__ __forceinline__ void sts2(float *p, float2 v) { *reinterpret_cast<float2 *>(p) = v; }
__device__ __forceinline__ float2 ldg2(const float *p) { return *reinterpret_cast<const float2 *>(p); }
__device__ __forceinline__ void stg2(float *p, float2 v) { *reinterpret_cast<float2 *>(p) = v; }

// Returns false when a bounded wait ran out (the error flag is then set); the
// same value in every thread of the CTA.
template <int PAR, int JM>
__device__ __forceinline__ bool wide_item(const Maps &maps, const Args &a, int tile_id, int i_begin, int i_end,
                                          bool first, int t, unsigned char *smem_raw) {
    unsigned char *smem = smem_raw + ((128u - (smem_u32(smem_raw) & 127u)) & 127u);
    float *hnb = (float *)(smem + NS * STAGE_BW);
    uint64_t *bar = (uint64_t *)(smem + NS * STAGE_BW + 2 * align128(HNW_B));
    volatile int *okflag = (volatile int *)(bar + NS);
    unsigned char *pf = (unsigned char *)(bar + NS) + 16;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int Nx = a.Nx, Ny = a.Ny;
    const int k0 = (tile_id % a.ntk) * TK, j0 = (tile_id / a.ntk) * TJ;
    if (i_begin >= i_end) return true;
    const int p0 = max(i_begin - 1, 0), q_last = min(i_end, Nx - 1);
    const size_t plane = (size_t)Ny * a.Nzp;

    if (first) line_update<PAR>(a, t);
    if (first && t > 0) record_probes<PAR>(a, t);
    if (tid == PROD) {
        for (int q = 0; q < NS; q++) mbar_init(&bar[q], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    // plasma flags of the item's planes: the block of either 8 x 32 half
    if (a.plasma && tid < PF_CAP && tid < i_end - p0) {
        const size_t r = (size_t)(p0 + tid) * a.ntiles + tile_id;
        pf[tid] = a.plasma[r] | a.plasma[r + 1];
    }
    __syncthreads();
    int issued = p0 - 1;
    auto issue = [&](int q) {
        const int slot = (q - p0) % NS;
        mbar_arm(&bar[slot], STAGE_TXW);
        tma4(smem + slot * STAGE_BW, &maps.F[PAR], k0 - 4, j0 - 1, q, 0, &bar[slot]);
    };
    if (tid == PROD) {
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        for (int q = p0; q <= q_last && q < p0 + NS; q++) {
            issue(q);
            issued = q;
        }
    }
    auto plasma_q = [&](int q) {
        if (!a.plasma) return true;
        const int r = q - p0;
        return r < PF_CAP ? pf[r] != 0
                          : (a.plasma[(size_t)q * a.ntiles + tile_id] | a.plasma[(size_t)q * a.ntiles + tile_id + 1]) != 0;
    };
    auto stage_ready = [&](int qq) {
        return qq > q_last || mbar_wait(&bar[(qq - p0) % NS], ((qq - p0) / NS) & 1);
    };

    // roles
    const bool tile = warp < TJ, row_halo = warp == TJ, col_halo = warp == TJ + 1 && lane < TJ;
    const int dj = tile ? warp : row_halo ? -1 : lane;
    const int dk = (tile || row_halo) ? 2 * lane : -1;
    const int j = j0 + dj, k = k0 + dk;
    const size_t col = tile ? (size_t)j * a.Nzp + k : 0;
    float2 Gk = make_float2(0.f, 0.f), G2k = Gk;
    if (tile) {
        Gk = make_float2(a.G[k], a.G[k + 1]);
        G2k = make_float2(a.G2[k], a.G2[k + 1]);
    }
    // plasma weight (and collision frequency) of the thread's cells, one plane ahead
    auto pf_load = [&](int qq, float2 &wq, float2 &nu) {
        if (!tile || qq >= Nx) return;
        const size_t ij = (size_t)qq * Ny + j;
        if (a.wq3) wq = ldg2(a.wq3 + (size_t)qq * plane + col);
        else wq.x = wq.y = a.wq2[ij];
        if (JM == 0) {
            if (a.nu3) nu = ldg2(a.nu3 + (size_t)qq * plane + col);
            else nu.x = nu.y = a.nu2[ij];
        }
    };
    float2 nwq = make_float2(0.f, 0.f), nnu = nwq;
    bool npl = plasma_q(p0);
    if (npl) pf_load(p0, nwq, nnu);

    if (tid == PROD) okflag[2] = (stage_ready(p0) && stage_ready(p0 + 1)) ? 1 : 0;
    __syncthreads();
    int fail_q = -1;
    if (!okflag[2]) fail_q = p0;

    float2 hyp = make_float2(0.f, 0.f), hzp = hyp, exp2v = hyp;  // previous plane's Hy, Hz, old Ex
    int slot = 0;
    size_t cg = (size_t)p0 * plane + col;
    const float c1h = a.c1h, chx = a.chx, chy = a.chy, chz = a.chz;
    for (int q = p0; fail_q < 0 && q < i_end; q++, cg += plane) {
        const float2 cwq = nwq, cnu = nnu;
        const bool pl = npl;
        npl = q + 1 < i_end && plasma_q(q + 1);
        if (npl) pf_load(q + 1, nwq, nnu);
        const int slot1 = slot == NS - 1 ? 0 : slot + 1;
        float *hn = hnb + (q & 1) * (align128(HNW_B) / 4);
        const float *sb = (const float *)(smem + slot * STAGE_BW);
        const float *sb1 = (const float *)(smem + slot1 * STAGE_BW);
        slot = slot1;
        const bool real = q >= i_begin;
        // component c of the stage: sb + c * (C_BW / 4)
        constexpr int CB = C_BW / 4;
        float2 e0 = make_float2(0.f, 0.f), e1 = e0, e2 = e0, hx = e0, hy = e0, hz = e0;
        float2 jx = e0, jy = e0, jz = e0;
        // The x-slab planes and the domain's x faces (uniform over the CTA):
        // the x-normal CPML terms of Hy, Hz, Ey, Ez (h_cell / e_cell in their
        // clean-tile form, same expression order), and the components the
        // faces do not update keep their old values.
        const int sxh = hslab(q, Nx, a.L, a.xshift);
        const bool xin = q < Nx - 1;
        const bool hpsi = a.dopml && sxh >= 0 && xin;
        const unsigned oxh = (unsigned)(max(sxh, 0) * Ny + j) * a.Nz + k;  // x-normal psi of (j, k)
        if (tile || row_halo) {
            e0 = lds2(sb + 0 * CB + EW(dj, dk));
            e1 = lds2(sb + 1 * CB + EW(dj, dk));
            e2 = lds2(sb + 2 * CB + EW(dj, dk));
            const float2 h0 = lds2(sb + 3 * CB + EW(dj, dk)), h2 = lds2(sb + 5 * CB + EW(dj, dk));
            const float2 e2j = lds2(sb + 2 * CB + EW(dj + 1, dk)), e0j = lds2(sb + 0 * CB + EW(dj + 1, dk));
            const float e1k = sb[1 * CB + EW(dj, dk + 2)];
            const float2 e1i = lds2(sb1 + 1 * CB + EW(dj, dk));
            hx.x = c1h * h0.x - (chy * (e2j.x - e2.x) - chz * (e1.y - e1.x));
            hx.y = c1h * h0.y - (chy * (e2j.y - e2.y) - chz * (e1k - e1.y));
            hz.x = c1h * h2.x - (chx * (e1i.x - e1.x) - chy * (e0j.x - e0.x));
            hz.y = c1h * h2.y - (chx * (e1i.y - e1.y) - chy * (e0j.y - e0.y));
            if (!xin) {
                hz = h2;
            } else if (hpsi) {  // zx psi: Hz -= c2h p
                const float B = a.tb->Bh[sxh], A = a.tb->Ahx[sxh], K = a.tb->Khx[sxh];
                const float dEy0 = e1i.x - e1.x, dEy1 = e1i.y - e1.y;
                const float p0 = B * a.Ph[PAR][4][oxh] + A * dEy0, p1 = B * a.Ph[PAR][4][oxh + 1] + A * dEy1;
                if (tile && real) {
                    a.Ph[PAR ^ 1][4][oxh] = p0;
                    a.Ph[PAR ^ 1][4][oxh + 1] = p1;
                }
                hz.x -= a.c2h * p0;
                hz.y -= a.c2h * p1;
                if (a.kappa_on) {
                    hz.x -= a.c2h * (K * dEy0);
                    hz.y -= a.c2h * (K * dEy1);
                }
            }
            sts2(hn + HNW(0, dj, dk), hx);
            sts2(hn + HNW(2, dj, dk), hz);
            if (tile) {
                const float2 h1 = lds2(sb + 4 * CB + EW(dj, dk));
                const float e0k = sb[0 * CB + EW(dj, dk + 2)];
                const float2 e2i = lds2(sb1 + 2 * CB + EW(dj, dk));
                hy.x = c1h * h1.x - (chz * (e0.y - e0.x) - chx * (e2i.x - e2.x));
                hy.y = c1h * h1.y - (chz * (e0k - e0.y) - chx * (e2i.y - e2.y));
                if (!xin) {
                    hy = h1;
                } else if (hpsi) {  // yx psi: Hy += c2h p
                    const float B = a.tb->Bh[sxh], A = a.tb->Ahx[sxh], K = a.tb->Khx[sxh];
                    const float dEz0 = e2i.x - e2.x, dEz1 = e2i.y - e2.y;
                    const float p0 = B * a.Ph[PAR][2][oxh] + A * dEz0, p1 = B * a.Ph[PAR][2][oxh + 1] + A * dEz1;
                    if (real) {
                        a.Ph[PAR ^ 1][2][oxh] = p0;
                        a.Ph[PAR ^ 1][2][oxh + 1] = p1;
                    }
                    hy.x += a.c2h * p0;
                    hy.y += a.c2h * p1;
                    if (a.kappa_on) {
                        hy.x += a.c2h * (K * dEz0);
                        hy.y += a.c2h * (K * dEz1);
                    }
                }
                sts2(hn + HNW(1, dj, dk), hy);
                if (real) {
                    stg2(a.H[PAR ^ 1][0] + cg, hx);
                    stg2(a.H[PAR ^ 1][1] + cg, hy);
                    stg2(a.H[PAR ^ 1][2] + cg, hz);
                    if (pl) {  // J of the previous step, lagged (source/meteor-fork.cpp:1539-1595)
                        jx = ldg2(a.J[0] + cg);
                        jy = ldg2(a.J[1] + cg);
                        jz = ldg2(a.J[2] + cg);
                        if (t > 0 && q >= 1 && xin) {
                            const float2 eyjm = lds2(sb + 1 * CB + EW(dj - 1, dk));
                            const float ezkm = sb[2 * CB + EW(dj, dk - 1)];
                            j_advance<JM>(a, a.lku, cwq.x, cnu.x, Gk.x, G2k.x, e0.x, e1.x, e2.x, exp2v.x, eyjm.x,
                                          ezkm, jx.x, jy.x, jz.x);
                            j_advance<JM>(a, a.lku, cwq.y, cnu.y, Gk.y, G2k.y, e0.y, e1.y, e2.y, exp2v.y, eyjm.y,
                                          e2.x, jx.y, jy.y, jz.y);
                        }
                    }
                }
            }
        } else if (col_halo) {  // H on the halo column k0 - 1: Hx and Hy
            const float ex = sb[0 * CB + EW(dj, -1)], ey = sb[1 * CB + EW(dj, -1)], ez = sb[2 * CB + EW(dj, -1)];
            const float h0 = sb[3 * CB + EW(dj, -1)], h1 = sb[4 * CB + EW(dj, -1)];
            hx.x = c1h * h0 - (chy * (sb[2 * CB + EW(dj + 1, -1)] - ez) - chz * (sb[1 * CB + EW(dj, 0)] - ey));
            const float dEz = sb1[2 * CB + EW(dj, -1)] - ez;
            hy.x = c1h * h1 - (chz * (sb[0 * CB + EW(dj, 0)] - ex) - chx * dEz);
            if (!xin) {
                hy.x = h1;
            } else if (hpsi) {
                const float p = a.tb->Bh[sxh] * a.Ph[PAR][2][oxh] + a.tb->Ahx[sxh] * dEz;
                hy.x += a.c2h * p;
                if (a.kappa_on) hy.x += a.c2h * (a.tb->Khx[sxh] * dEz);
            }
            hn[HNW(0, dj, -1)] = hx.x;
            hn[HNW(1, dj, -1)] = hy.x;
        }
        // one CTA barrier per plane: the new-H plane is complete; the stage of
        // plane q+2 has landed; the producer refills plane q-1's slot
        if (tid == PROD) okflag[q & 1] = stage_ready(q + 2) ? 1 : 0;
        __syncthreads();
        if (!okflag[q & 1]) {
            fail_q = q + 2;
            break;
        }
        if (tid == PROD && q > p0 && q - 1 + NS <= q_last) {
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            issue(q - 1 + NS);
            issued = q - 1 + NS;
        }
        if (tile) {
            if (real) {
                const float c1 = a.c1e0, c2 = a.c2e0, cex = a.cex, cey = a.cey, cez = a.cez;
                const float2 hzj = lds2(hn + HNW(2, dj - 1, dk)), hxj = lds2(hn + HNW(0, dj - 1, dk));
                const float hykm = hn[HNW(1, dj, dk - 1)], hxkm = hn[HNW(0, dj, dk - 1)];
                float2 ex, ey, ez;
                ex.x = c1 * e0.x + (cey * (hz.x - hzj.x) - cez * (hy.x - hykm)) - c2 * jx.x;
                ex.y = c1 * e0.y + (cey * (hz.y - hzj.y) - cez * (hy.y - hy.x)) - c2 * jx.y;
                ey.x = c1 * e1.x + (cez * (hx.x - hxkm) - cex * (hz.x - hzp.x)) - c2 * jy.x;
                ey.y = c1 * e1.y + (cez * (hx.y - hx.x) - cex * (hz.y - hzp.y)) - c2 * jy.y;
                ez.x = c1 * e2.x + (cex * (hy.x - hyp.x) - cey * (hx.x - hxj.x)) - c2 * jz.x;
                ez.y = c1 * e2.y + (cex * (hy.y - hyp.y) - cey * (hx.y - hxj.y)) - c2 * jz.y;
                if (q < 1 || !xin) {  // x faces: Ey, Ez not updated; Ex not at Nx - 1
                    ey = e1;
                    ez = e2;
                    if (!xin) ex = e0;
                } else {
                    const int sxe = a.dopml ? eslab(q, Nx, a.L, a.xshift) : -1;
                    if (sxe >= 0) {  // yx and zx psi: Ey -= c2 p, Ez += c2 p
                        const float B = a.tb->Be[sxe], A = a.tb->Aex[sxe], K = a.tb->Kex[sxe];
                        const unsigned oxe = (unsigned)(sxe * Ny + j) * a.Nz + k;
                        const float dHz0 = hz.x - hzp.x, dHz1 = hz.y - hzp.y;
                        const float dHy0 = hy.x - hyp.x, dHy1 = hy.y - hyp.y;
                        const float py0 = B * a.Pe[2][oxe] + A * dHz0, py1 = B * a.Pe[2][oxe + 1] + A * dHz1;
                        const float pz0 = B * a.Pe[4][oxe] + A * dHy0, pz1 = B * a.Pe[4][oxe + 1] + A * dHy1;
                        a.Pe[2][oxe] = py0;
                        a.Pe[2][oxe + 1] = py1;
                        a.Pe[4][oxe] = pz0;
                        a.Pe[4][oxe + 1] = pz1;
                        ey.x -= a.c2e0 * py0;
                        ey.y -= a.c2e0 * py1;
                        ez.x += a.c2e0 * pz0;
                        ez.y += a.c2e0 * pz1;
                        if (a.kappa_on) {
                            ey.x -= a.c2e0 * (K * dHz0);
                            ey.y -= a.c2e0 * (K * dHz1);
                            ez.x += a.c2e0 * (K * dHy0);
                            ez.y += a.c2e0 * (K * dHy1);
                        }
                    }
                }
                stg2(a.E[PAR ^ 1][0] + cg, ex);
                stg2(a.E[PAR ^ 1][1] + cg, ey);
                stg2(a.E[PAR ^ 1][2] + cg, ez);
                if (pl) {
                    stg2(a.J[0] + cg, jx);
                    stg2(a.J[1] + cg, jy);
                    stg2(a.J[2] + cg, jz);
                }
            }
            exp2v = e0;
            hyp = hy;
            hzp = hz;
        }
    }
    if (fail_q >= 0 && tid == PROD) {
        atomicOr(a.err, 1u);
        // Let the copies already issued land (bounded) before the CTA exits.
        for (int qq = fail_q; qq <= issued; qq++) {
            const int sl = (qq - p0) % NS;
            const unsigned pp = ((qq - p0) / NS) & 1;
            const uint64_t t0 = globaltimer();
            while (!mbar_test(&bar[sl], pp) && globaltimer() - t0 < 200000000ull) {
            }
        }
    }
    return fail_q < 0;
}

template <int PAR, int JM>
__global__ void __launch_bounds__(NTHREADS, 2)
    k_fp32_step_wide(const __grid_constant__ Maps maps, const __grid_constant__ Args a, int t) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    const bool first = blockIdx.x == 0 && blockIdx.y == 0 && blockIdx.z == 0;
    const int ib = a.xbeg + (int)blockIdx.z * a.chunk;
    wide_item<PAR, JM>(maps, a, a.tile_order[blockIdx.x], ib, min(a.xend, ib + a.chunk), first, t, smem_raw);
}

// ---------------------------------------------------------------------------
// Batched form: many simulations advance one time step per launch.  Their Args
// sit in constant-bank slots, their TMA descriptors in global memory.  A
// persistent grid (a few CTAs per SM) pulls work items -- (simulation, tile,
// x-chunk) -- from a device queue until it is empty; items of boundary tiles
// come first.  A simulation past its step count keeps its slot but gets no
// work.  k_batch_advance then moves every simulation to its next step and
// resets the queue, so K steps replay as one CUDA graph.
constexpr int kMaxBatch = 56;  // 56 x 1080-byte Args in the 64 KB constant bank
__constant__ Args c_jobs[kMaxBatch];

// A work item of the batch: simulation slot `job`, tile `tile` over the planes
// [ib, ie), marched as `mode` (MARCH_GENERAL, MARCH_FAST or MARCH_SLAB);
// `first` advances the simulation's incident line and records its probes.
struct BatchItem {
    int job, tile;
    unsigned short ib, ie;
    unsigned char mode, first, yz, pad;  // yz: MARCH_SLAB items' axis class (slab_view)
};

// KIND: 0, every item takes the general path; 1, a batch whose members all
// qualify for the slab march (Fp32Sim::batch_class), items on the fast path
// (8 x 32 tiles) or the slab march; 2, the same members with their interior
// tiles paired into 8 x 64 tiles on the wide path (two cells per thread).
// (One kernel holding every path spills.)  A CTA that moves from one
// shared-memory layout to the other first invalidates the mbarriers of the
// layout it leaves: the next item's stages overwrite that memory.
enum : int { MARCH_WIDE = 3 };
template <int PAR, int JM, int KIND>
__global__ void __launch_bounds__(NTHREADS, (JM == 2 || KIND == 2) ? 2 : 3)
    k_fp32_batch(const BatchItem *__restrict__ items, const int *__restrict__ n_items, int *next,
                 const Maps *__restrict__ maps, const Maps *__restrict__ mapsw, const int *__restrict__ job_t,
                 const int *__restrict__ job_end) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ int s_item;
    unsigned char *sm = smem_raw + ((128u - (smem_u32(smem_raw) & 127u)) & 127u);
    uint64_t *bar_n = (uint64_t *)(sm + NS * STAGE_B + 2 * align128(HN_B));     // run_item's layout
    uint64_t *bar_w = (uint64_t *)(sm + NS * STAGE_BW + 2 * align128(HNW_B));   // wide_item's layout
    int last = 0;  // layout of the previous item: 0 none, 1 run_item, 2 wide_item
    const int n = *n_items;
    for (;;) {
        __syncthreads();  // everyone has read s_item of the previous round
        if (threadIdx.x == 0) s_item = atomicAdd(next, 1);
        __syncthreads();
        const int it = s_item;
        if (it >= n) break;
        const BatchItem w = items[it];
        const int t = job_t[w.job];
        if (t >= job_end[w.job]) continue;
        const Args &a = c_jobs[w.job];
        if (threadIdx.x == PROD && last != 0) {
            uint64_t *b = last == 1 ? bar_n : bar_w;
            for (int q = 0; q < NS; q++)
                asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(smem_u32(&b[q])) : "memory");
        }
        bool ok = true;
        if constexpr (KIND == 2) {
            if (w.mode == MARCH_WIDE) {
                ok = wide_item<PAR, JM>(mapsw[w.job], a, w.tile, w.ib, w.ie, w.first != 0, t, smem_raw);
                last = 2;
            } else {
                const Maps &mp = maps[w.job];
                const bool f = w.first != 0;
                if (w.yz == 1) ok = run_item<PAR, JM, MARCH_SLAB, true, 1>(mp, a, w.tile, w.ib, w.ie, f, t, 0, smem_raw, false);
                else if (w.yz == 2) ok = run_item<PAR, JM, MARCH_SLAB, true, 2>(mp, a, w.tile, w.ib, w.ie, f, t, 0, smem_raw, false);
                else ok = run_item<PAR, JM, MARCH_SLAB>(mp, a, w.tile, w.ib, w.ie, f, t, 0, smem_raw, false);
                last = 1;
            }
        } else if constexpr (KIND == 1) {
            const Maps &mp = maps[w.job];
            const bool f = w.first != 0;
            if (w.mode == MARCH_FAST)
                ok = run_item<PAR, JM, MARCH_FAST>(mp, a, w.tile, w.ib, w.ie, f, t, 0, smem_raw, false);
            // (three CTAs per SM: no registers for the psi prefetch)
            else if (w.yz == 0) ok = run_item<PAR, JM, MARCH_SLAB, false, 0>(mp, a, w.tile, w.ib, w.ie, f, t, 0, smem_raw, false);
            else if (w.yz == 1) ok = run_item<PAR, JM, MARCH_SLAB, false, 1>(mp, a, w.tile, w.ib, w.ie, f, t, 0, smem_raw, false);
            else if (w.yz == 2) ok = run_item<PAR, JM, MARCH_SLAB, false, 2>(mp, a, w.tile, w.ib, w.ie, f, t, 0, smem_raw, false);
            else ok = run_item<PAR, JM, MARCH_SLAB, false>(mp, a, w.tile, w.ib, w.ie, f, t, 0, smem_raw, false);
            last = 1;
        } else {
            ok = run_item<PAR, JM>(maps[w.job], a, w.tile, w.ib, w.ie, w.first != 0, t, 0, smem_raw, false);
            last = 1;
        }
        if (!ok) break;
    }
}

__global__ void k_batch_advance(int *job_t, const int *job_end, int njobs, int *next) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j < njobs && job_t[j] < job_end[j]) job_t[j] += 1;
    if (j == 0) *next = 0;
}

// ---------------------------------------------------------------------------

// The running DFT on the Huygens surface (source/meteor-2.1.cpp:942-992,
// 1386-1438), in two kernels.  Each step, k_fp32_ntf (or, in a batch,
// k_batch_post) copies the face values the sums need from the state pass t
// wrote (set `cur`) into slot `slot` of a ring of kNtfRing steps: per face
// cell, the two tangential H components at the face node and at the node
// behind it, and the two tangential E components (six floats, component-major
// for coalescing).  Every kNtfRing steps, at the end of every advance, and at
// a batch member's last step, k_fp32_ntf_flush (k_batch_flush) adds the
// ring's steps to the FP64 sums: per cell and frequency it forms the
// reference's terms -- H averaged over the two nodes, E at the face node,
// signs per face, times the step's phase -- in
// double-float arithmetic (value pairs hi + lo of FP32 numbers: the H average
// kept exact by a two-sum, the phase split into two floats, each product
// kept with its exact rounding error by an FMA), sums them over the ring's
// steps with a compensated two-sum accumulation, and adds the result to the
// FP64 sums once.  The terms carry about 44 bits, so the sums match the
// per-step FP64 accumulation to about 1e-13 relative; the sums'
// read-modify-writes and their FP64 arithmetic (a slow pipe on this part)
// are paid once per ring instead of every step.
constexpr int kNtfRing = 8;
struct NtfFace {
    int arr;     // first of the face's four sum arrays (Args::ntf)
    float sgn;   // +1 on the front, top and left faces, -1 opposite
    size_t c, s; // face node offset, offset to the node behind it
    size_t r;    // cell index within the face (row of the sum arrays)
};
__device__ __forceinline__ NtfFace ntf_face(const Args &a, size_t q) {
    const int Nx = a.Nx, Ny = a.Ny, Nz = a.Nz, nb = a.ntfb;
    const size_t fx = (size_t)Ny * Nz, fy = (size_t)Nx * Nz, fz = (size_t)Nx * Ny;
    const size_t sJ = a.Nzp, sI = (size_t)Ny * a.Nzp;
    NtfFace f;
    size_t r = q;
    if (r < 2 * fx) {  // x faces: front (i = nb), back (i = Nx - nb); r = j * Nz + k
        const bool back = r >= fx;
        if (back) r -= fx;
        const int i = back ? Nx - nb : nb, j = (int)((unsigned)r / (unsigned)Nz), k = (int)((unsigned)r % (unsigned)Nz);
        f.c = i * sI + j * sJ + k;
        f.s = sI;
        f.arr = back ? 4 : 0;
        f.sgn = back ? -1.f : 1.f;
    } else if ((r -= 2 * fx) < 2 * fy) {  // y faces: top (j = Ny - nb), bottom (j = nb); r = i * Nz + k
        const bool bottom = r >= fy;
        if (bottom) r -= fy;
        const int j = bottom ? nb : Ny - nb, i = (int)((unsigned)r / (unsigned)Nz), k = (int)((unsigned)r % (unsigned)Nz);
        f.c = i * sI + j * sJ + k;
        f.s = sJ;
        f.arr = bottom ? 12 : 8;
        f.sgn = bottom ? -1.f : 1.f;
    } else {  // z faces: left (k = nb), right (k = Nz - nb); r = i * Ny + j
        r -= 2 * fy;
        const bool right = r >= fz;
        if (right) r -= fz;
        const int k = right ? Nz - nb : nb, i = (int)((unsigned)r / (unsigned)Ny), j = (int)((unsigned)r % (unsigned)Ny);
        f.c = i * sI + j * sJ + k;
        f.s = 1;
        f.arr = right ? 20 : 16;
        f.sgn = right ? -1.f : 1.f;
    }
    f.r = r;
    return f;
}
__device__ __forceinline__ void ntf_stash(const Args &a, int cur, float *__restrict__ ring, int slot, size_t q0,
                                          size_t dq) {
    const size_t fx = (size_t)a.Ny * a.Nz, fy = (size_t)a.Nx * a.Nz, fz = (size_t)a.Nx * a.Ny;
    const size_t total = 2 * (fx + fy + fz);
    float *const r = ring + (size_t)slot * 6 * total;
    for (size_t q = q0; q < total; q += dq) {
        const NtfFace f = ntf_face(a, q);
        // (Ha, Hb, Ea, Eb): x faces (Hz, Hy, Ey, Ez), y faces (Hz, Hx, Ex, Ez), z faces (Hy, Hx, Ex, Ey)
        const int xf = f.arr < 8, yf = f.arr >= 8 && f.arr < 16;
        const float *Ha = a.H[cur][xf || yf ? 2 : 1], *Hb = a.H[cur][xf ? 1 : 0];
        const float *Ea = a.E[cur][xf ? 1 : 0], *Eb = a.E[cur][xf || yf ? 2 : 1];
        r[q] = Ha[f.c];
        r[total + q] = Ha[f.c - f.s];
        r[2 * total + q] = Hb[f.c];
        r[3 * total + q] = Hb[f.c - f.s];
        r[4 * total + q] = Ea[f.c];
        r[5 * total + q] = Eb[f.c];
    }
}
__global__ void __launch_bounds__(256) k_fp32_ntf(const __grid_constant__ Args a, int cur, float *__restrict__ ring,
                                                  int slot) {
    ntf_stash(a, cur, ring, slot, (size_t)blockIdx.x * blockDim.x + threadIdx.x, (size_t)gridDim.x * blockDim.x);
}
// s + y = t + e exactly (Knuth's two-sum).
__device__ __forceinline__ float two_sum(float s, float y, float &e) {
    const float t = __fadd_rn(s, y), bp = __fsub_rn(t, s);
    e = __fadd_rn(__fsub_rn(s, __fsub_rn(t, bp)), __fsub_rn(y, bp));
    return t;
}
// Adds (vh + vl) * (ph + pl) to the compensated sum (s, c); the product's
// high part is exact up to its rounding error, which an FMA recovers.
__device__ __forceinline__ void df_mac(float &s, float &c, float vh, float vl, float ph, float pl) {
    const float p = __fmul_rn(vh, ph);
    const float pe = __fmaf_rn(vh, ph, -p);
    float e;
    s = two_sum(s, p, e);
    c += e + (pe + (vh * pl + vl * ph));
}
// Ring slots 0 .. count-1 hold steps t0 .. t0 + count - 1.  The terms:
// arrays arr+2, arr+3 take (sgn * H_a, -sgn * H_b) and arrays
// arr, arr+1 take (-sgn * E_b, sgn * E_a), each times (cos, sin) of the
// step's phase; phase4 holds per (step, frequency) the phase's FP32 high
// parts and the FP32 remainders.
__device__ __forceinline__ void ntf_flush_cells(const Args &a, const float *__restrict__ ring,
                                                const float4 *__restrict__ phase4, int t0, int count, size_t q0,
                                                size_t dq) {
    const int nf = a.nntf;
    const size_t fx = (size_t)a.Ny * a.Nz, fy = (size_t)a.Nx * a.Nz, fz = (size_t)a.Nx * a.Ny;
    const size_t total = 2 * (fx + fy + fz), slot = 6 * total;
    for (size_t q = q0; q < total; q += dq) {
        const NtfFace f = ntf_face(a, q);
        const size_t base = f.r * 2 * (size_t)nf;
        for (int m = 0; m < nf; m++) {
            float s[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f}, c[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
            for (int u = 0; u < count; u++) {
                const float *r = ring + u * slot + q;
                // the H averages as exact pairs: 0.5 (x + y) = 0.5 t + 0.5 e
                float ea_, eb_;
                const float ta = two_sum(r[0], r[total], ea_), tb = two_sum(r[2 * total], r[3 * total], eb_);
                const float g = f.sgn;
                const float vh[4] = {g * 0.5f * ta, -g * 0.5f * tb, -g * r[5 * total], g * r[4 * total]};
                const float vl[4] = {g * 0.5f * ea_, -g * 0.5f * eb_, 0.f, 0.f};
                const float4 p = phase4[(size_t)(t0 + u) * nf + m];
#pragma unroll
                for (int w = 0; w < 4; w++) {
                    df_mac(s[2 * w], c[2 * w], vh[w], vl[w], p.x, p.z);
                    df_mac(s[2 * w + 1], c[2 * w + 1], vh[w], vl[w], p.y, p.w);
                }
            }
            const int arr[4] = {f.arr + 2, f.arr + 3, f.arr, f.arr + 1};
#pragma unroll
            for (int w = 0; w < 4; w++) {
                double2 *d = (double2 *)(a.ntf[arr[w]] + base) + m;
                double2 x = *d;
                x.x += (double)s[2 * w] + (double)c[2 * w];
                x.y += (double)s[2 * w + 1] + (double)c[2 * w + 1];
                *d = x;
            }
        }
    }
}
__global__ void __launch_bounds__(256) k_fp32_ntf_flush(const __grid_constant__ Args a, const float *__restrict__ ring,
                                                        const float4 *__restrict__ phase4, int t0, int count) {
    ntf_flush_cells(a, ring, phase4, t0, count, (size_t)blockIdx.x * blockDim.x + threadIdx.x,
                    (size_t)gridDim.x * blockDim.x);
}

// The oblique TF/SF corrections as a pass of their own (single simulations
// without a plate or a conducting sphere).  The step kernel updated H and E
// of pass PAR without them.  They are linear in the fields' update, so each
// cell of the band around the TF/SF surface adds here its H correction dH,
// and to E its own correction plus the curl of the neighbouring dH with the
// E update's coefficients -- what the inline form adds, up to rounding.  The
// band is every cell of [b1-1, b2]^3 with a coordinate in {b1-1, b1, b2-1, b2}
// (each enumerated once), which holds every node a correction reaches; with
// tfsf_gap >= 2 it lies outside the CPML slabs, so no psi term is involved.
// The line values are the ones of the pass's start (set PAR; the pass wrote
// the next line into the other set).  On record steps the slice entries of
// band cells get the same increments.
// One cell of the TF/SF band: its H correction dH, and its E correction plus
// the curl of the dH of the cell and of its -x, -y, -z neighbours, added to
// the new state (and to the slices on record steps).  Bit AX of MASK says
// that crossing terms along axis AX can be nonzero for the cell and those
// neighbours; the terms of the other axes are exactly zero there and are not
// evaluated (obl_corr_m), which leaves the sums unchanged.
template <int PAR, bool IS_E, int C, int MASK>
__device__ __forceinline__ float obl_corr_m(const Args &a, int i, int j, int k) {
    constexpr int A1 = (C + 1) % 3, A2 = (C + 2) % 3;
    float v1 = 0.f, v2 = 0.f;
    if constexpr ((MASK >> A1) & 1) v1 = obl_axis<PAR, IS_E, C, A1>(a, i, j, k);
    if constexpr ((MASK >> A2) & 1) v2 = obl_axis<PAR, IS_E, C, A2>(a, i, j, k);
    return __fadd_rn(v1, v2);
}
template <int PAR, int MASK>
__device__ __forceinline__ void tfsf_cell(const Args &a, int record, int i, int j, int k, size_t plane) {
    const float hx = obl_corr_m<PAR, false, 0, MASK>(a, i, j, k);
    const float hy = obl_corr_m<PAR, false, 1, MASK>(a, i, j, k);
    const float hz = obl_corr_m<PAR, false, 2, MASK>(a, i, j, k);
    // E's own correction plus the E update's curl of the neighbouring dH
    // (explicitly rounded: see obl_axis)
    auto curl = [](float c1, float d1, float c2, float d2, float own) {
        return __fadd_rn(__fsub_rn(__fmul_rn(c1, d1), __fmul_rn(c2, d2)), own);
    };
    const float ex = curl(a.cey, __fsub_rn(hz, obl_corr_m<PAR, false, 2, MASK>(a, i, j - 1, k)), a.cez,
                          __fsub_rn(hy, obl_corr_m<PAR, false, 1, MASK>(a, i, j, k - 1)),
                          obl_corr_m<PAR, true, 0, MASK>(a, i, j, k));
    const float ey = curl(a.cez, __fsub_rn(hx, obl_corr_m<PAR, false, 0, MASK>(a, i, j, k - 1)), a.cex,
                          __fsub_rn(hz, obl_corr_m<PAR, false, 2, MASK>(a, i - 1, j, k)),
                          obl_corr_m<PAR, true, 1, MASK>(a, i, j, k));
    const float ez = curl(a.cex, __fsub_rn(hy, obl_corr_m<PAR, false, 1, MASK>(a, i - 1, j, k)), a.cey,
                          __fsub_rn(hx, obl_corr_m<PAR, false, 0, MASK>(a, i, j - 1, k)),
                          obl_corr_m<PAR, true, 2, MASK>(a, i, j, k));
    const size_t c = (size_t)i * plane + (size_t)j * a.Nzp + k;
    if (hx != 0.f) a.H[PAR ^ 1][0][c] += hx;
    if (hy != 0.f) a.H[PAR ^ 1][1][c] += hy;
    if (hz != 0.f) a.H[PAR ^ 1][2][c] += hz;
    if (ex != 0.f) a.E[PAR ^ 1][0][c] += ex;
    if (ey != 0.f) a.E[PAR ^ 1][1][c] += ey;
    if (ez != 0.f) a.E[PAR ^ 1][2][c] += ez;
    if (record) {  // slices written by the pass (source/meteor-2.1.cpp:996-1013, 1322-1340)
        const int Nx = a.Nx, Ny = a.Ny, Nz = a.Nz;
        const size_t oz = 0, oy = 2 * (size_t)Nx * Ny, ox = oy + 2 * (size_t)Nx * Nz;
        if (k == a.ssz) {
            a.slE[oz + (size_t)i * Ny + j] += ey;
            a.slE[oz + (size_t)Nx * Ny + (size_t)i * Ny + j] += ez;
            if (j < Ny - 1) {
                a.slH[oz + (size_t)i * Ny + j] += hy;
                a.slH[oz + (size_t)Nx * Ny + (size_t)i * Ny + j] += hz;
            }
        }
        if (j == a.ssy) {
            a.slE[oy + (size_t)i * Nz + k] += ey;
            a.slE[oy + (size_t)Nx * Nz + (size_t)i * Nz + k] += ez;
            if (k < Nz - 1) {
                a.slH[oy + (size_t)i * Nz + k] += hy;
                a.slH[oy + (size_t)Nx * Nz + (size_t)i * Nz + k] += hz;
            }
        }
        if (i == a.ssx) {
            a.slE[ox + (size_t)j * Nz + k] += ey;
            a.slE[ox + (size_t)Ny * Nz + (size_t)j * Nz + k] += ez;
            if (j < Ny - 1 && k < Nz - 1) {
                a.slH[ox + (size_t)j * Nz + k] += hy;
                a.slH[ox + (size_t)Ny * Nz + (size_t)j * Nz + k] += hz;
            }
        }
    }
}

template <int PAR>
__device__ __forceinline__ void tfsf_band(const Args &a, int record, int r0, int dr, int c0, int dc) {
    const int bx1 = a.bx1, bx2 = a.bx2, by1 = a.by1, by2 = a.by2, bz1 = a.bz1, bz2 = a.bz2;
    const int Jr = by2 - by1 + 2, Kr = bz2 - bz1 + 2, Ir2 = max(bx2 - bx1 - 2, 0), Jr2 = by2 - by1 - 2;
    const size_t plane = (size_t)a.Ny * a.Nzp;
    auto pick = [](int b1, int b2, int s) { return s == 0 ? b1 - 1 : s == 1 ? b1 : s == 2 ? b2 - 1 : b2; };
    // The band as rows, each cell once: the x layers' rows (4 x Jr rows along
    // j, cells along k over [bz1 - 1, bz2]), the y layers' rows (4 x Ir2
    // along i, cells along k) and the z layers' rows (4 x Ir2 along i, cells
    // along j over [by1 + 1, by2 - 2]).  Rows r0, r0 + dr, ... and a row's
    // cells c0, c0 + dc, ...: no division in the indexing.
    const int rX = 4 * Jr, rY = 4 * Ir2, rZ = 4 * Ir2;
    auto layer = [](int r, int n) { return r < n ? 0 : r < 2 * n ? 1 : r < 3 * n ? 2 : 3; };
    // Crossing terms along an axis need the cell's (or its -1 neighbour's)
    // index on that axis in {b1 - 1, b1, b2 - 1, b2}: the x layers away from
    // their y and z edges, the y layers away from their z edges and every z
    // layer cell need one axis's terms only.
    for (int r = r0; r < rX + rY + rZ; r += dr) {
        if (r < rX) {
            const int l = layer(r, Jr);
            const int i = pick(bx1, bx2, l), j = by1 - 1 + (r - l * Jr);
            const bool yedge = j <= by1 || j >= by2 - 1;
            for (int c = c0; c < Kr; c += dc) {
                const int k = bz1 - 1 + c;
                const bool zedge = k <= bz1 || k >= bz2 - 1;
                if (yedge && zedge) tfsf_cell<PAR, 7>(a, record, i, j, k, plane);
                else if (yedge) tfsf_cell<PAR, 3>(a, record, i, j, k, plane);
                else if (zedge) tfsf_cell<PAR, 5>(a, record, i, j, k, plane);
                else tfsf_cell<PAR, 1>(a, record, i, j, k, plane);
            }
        } else if (r < rX + rY) {
            const int rr = r - rX, l = layer(rr, Ir2);
            const int j = pick(by1, by2, l), i = bx1 + 1 + (rr - l * Ir2);
            for (int c = c0; c < Kr; c += dc) {
                const int k = bz1 - 1 + c;
                if (k <= bz1 || k >= bz2 - 1) tfsf_cell<PAR, 6>(a, record, i, j, k, plane);
                else tfsf_cell<PAR, 2>(a, record, i, j, k, plane);
            }
        } else {
            const int rr = r - rX - rY, l = layer(rr, Ir2);
            const int k = pick(bz1, bz2, l), i = bx1 + 1 + (rr - l * Ir2);
            for (int c = c0; c < Jr2; c += dc) tfsf_cell<PAR, 4>(a, record, i, by1 + 1 + c, k, plane);
        }
    }
}
// The same band as one flat index space (one cell per thread and stride,
// divisions in the indexing): the batch follow-up kernel's form, whose
// members' bands are small (on 64-256-cell grids the row form left most of
// a block idle and needed 109 registers there: a tick 6 % slower).
template <int PAR>
__device__ __forceinline__ void tfsf_band_flat(const Args &a, int record, size_t q0, size_t dq) {
    const int bx1 = a.bx1, bx2 = a.bx2, by1 = a.by1, by2 = a.by2, bz1 = a.bz1, bz2 = a.bz2;
    const int Jr = by2 - by1 + 2, Kr = bz2 - bz1 + 2, Ir2 = bx2 - bx1 - 2, Jr2 = by2 - by1 - 2;
    const size_t nX = 4 * (size_t)Jr * Kr, nY = 4 * (size_t)Ir2 * Kr, nZ = 4 * (size_t)Ir2 * Jr2;
    const size_t plane = (size_t)a.Ny * a.Nzp;
    auto pick = [](int b1, int b2, int s) { return s == 0 ? b1 - 1 : s == 1 ? b1 : s == 2 ? b2 - 1 : b2; };
    // band sizes stay far below 2^31 (four face layers), so the index
    // decomposition runs in 32-bit arithmetic
    const unsigned uKr = (unsigned)Kr, uJr2 = (unsigned)Jr2, aX = (unsigned)Jr * uKr,
                   aY = (unsigned)Ir2 * uKr, aZ = (unsigned)Ir2 * uJr2;
    for (size_t q = q0; q < nX + nY + nZ; q += dq) {
        int i, j, k;
        if (q < nX) {
            const unsigned u = (unsigned)q, r = u % aX;
            i = pick(bx1, bx2, (int)(u / aX));
            j = by1 - 1 + (int)(r / uKr);
            k = bz1 - 1 + (int)(r % uKr);
        } else if (q < nX + nY) {
            const unsigned u = (unsigned)(q - nX), r = u % aY;
            j = pick(by1, by2, (int)(u / aY));
            i = bx1 + 1 + (int)(r / uKr);
            k = bz1 - 1 + (int)(r % uKr);
        } else {
            const unsigned u = (unsigned)(q - nX - nY), r = u % aZ;
            k = pick(bz1, bz2, (int)(u / aZ));
            i = bx1 + 1 + (int)(r / uJr2);
            j = by1 + 1 + (int)(r % uJr2);
        }
        // Crossing terms along an axis need the cell's (or its -1
        // neighbour's) index on that axis in {b1 - 1, b1, b2 - 1, b2}.  The x
        // layers span j, k over [b1 - 1, b2], the y layers k over
        // [bz1 - 1, bz2] with i inside, the z layers i and j inside.
        if (q < nX) {
            const bool yedge = j <= by1 || j >= by2 - 1, zedge = k <= bz1 || k >= bz2 - 1;
            if (yedge && zedge) tfsf_cell<PAR, 7>(a, record, i, j, k, plane);
            else if (yedge) tfsf_cell<PAR, 3>(a, record, i, j, k, plane);
            else if (zedge) tfsf_cell<PAR, 5>(a, record, i, j, k, plane);
            else tfsf_cell<PAR, 1>(a, record, i, j, k, plane);
        } else if (q < nX + nY) {
            if (k <= bz1 || k >= bz2 - 1) tfsf_cell<PAR, 6>(a, record, i, j, k, plane);
            else tfsf_cell<PAR, 2>(a, record, i, j, k, plane);
        } else {
            tfsf_cell<PAR, 4>(a, record, i, j, k, plane);
        }
    }
}
template <int PAR>
__global__ void __launch_bounds__(256) k_fp32_tfsf(const __grid_constant__ Args a, int record) {
    tfsf_band<PAR>(a, record, blockIdx.x, gridDim.x, threadIdx.x, blockDim.x);
}

// The same follow-up work for every member of a batch after its tick's pass
// PAR (no record steps in a batch): grid row y = the member's slot.  Empty,
// removed and finished slots (t >= end) return at once.
template <int PAR>
__global__ void __launch_bounds__(256) k_batch_post(const int *__restrict__ job_t, const int *__restrict__ job_end) {
    const int q = blockIdx.y;
    const int t = job_t[q];
    if (t >= job_end[q]) return;
    const Args &a = c_jobs[q];
    const size_t q0 = (size_t)blockIdx.x * blockDim.x + threadIdx.x, dq = (size_t)gridDim.x * blockDim.x;
    if (a.oblique && !a.obl_inline) tfsf_band_flat<PAR>(a, 0, q0, dq);
    if (a.nntf > 0 && a.ntf_ring) ntf_stash(a, PAR ^ 1, a.ntf_ring, t % kNtfRing, q0, dq);
}
// After k_batch_post: a member whose tick filled its DFT ring (step t with
// t % kNtfRing the last slot) or reached its last step adds the ring's steps
// to its FP64 sums, as a single simulation's k_fp32_ntf_flush does.
__global__ void __launch_bounds__(256) k_batch_flush(const int *__restrict__ job_t, const int *__restrict__ job_end) {
    const int q = blockIdx.y;
    const int t = job_t[q], end = job_end[q];
    if (t >= end) return;
    const Args &a = c_jobs[q];
    if (a.nntf <= 0 || !a.ntf_ring) return;
    const int u = t % kNtfRing;
    if (u != kNtfRing - 1 && t + 1 != end) return;
    ntf_flush_cells(a, a.ntf_ring, a.phase4, t - u, u + 1, (size_t)blockIdx.x * blockDim.x + threadIdx.x,
                    (size_t)gridDim.x * blockDim.x);
}

// ---------------------------------------------------------------------------
// CPML band (Args::band).  The pass updates every cell as an interior one; the
// band kernels then recompute, from the state the pass read, the cells with a
// coordinate in the first or last `w` indices of an axis (w = L + 1 with the
// CPML, else 1): the CPML slabs of H and E and the domain edges.  They use
// h_cell and e_cell with the CPML corrections, so every cell gets the same
// arithmetic as in the pass's general path, and the results are those of a
// pass that makes the corrections itself.  Interior cells never read a band
// H value (E at index n reads H at n and n-1, and H at L-1 and N-L-1 are the
// first band H cells), so only band cells are rewritten.  The H psi is double
// buffered and the pass does not touch the E psi, so the recomputation reads
// the psi of the previous step.
//
// Work unit: one warp, up to 32 cells of one (i, j) row, from a table built
// at set-up (consecutive units are consecutive segments, so the grid sweeps
// memory in order): rows (i in band, any j) and (interior i, j in band) in
// 32-cell segments along k; rows (interior i, interior j) over their 2w band
// cells k in [0, w) and [Nz-w, Nz) (the band-list flag), in 32-cell segments
// of that list.
template <class F>
__device__ __forceinline__ void for_band_cells(const Args &a, F &&f) {
    const int lane = threadIdx.x & 31, w = a.dopml ? a.L + 1 : 1;
    for (int u = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; u < a.n_band_units;
         u += (gridDim.x * blockDim.x) >> 5) {
        const int2 e = a.band_units[u];
        const int i = e.x & 0xffff, j = (unsigned)e.x >> 16, m = (e.y & 0xffff) + lane, n = (e.y >> 16) & 0xff;
        if (lane >= n) continue;
        f(i, j, (e.y >> 24) ? (m < w ? m : a.Nz - 2 * w + m) : m);
    }
}

// Record-step slice entries of a recomputed cell (the pass's layout and
// conditions, general path).
__device__ __forceinline__ void band_slices_e(const Args &a, int i, int j, int k, float ey, float ez_slice) {
    const int Nx = a.Nx, Ny = a.Ny, Nz = a.Nz;
    const size_t oz = 0, oy = 2 * (size_t)Nx * Ny, ox = oy + 2 * (size_t)Nx * Nz;
    if (k == a.ssz) {
        a.slE[oz + (size_t)i * Ny + j] = ey;
        a.slE[oz + (size_t)Nx * Ny + (size_t)i * Ny + j] = ez_slice;
    }
    if (j == a.ssy) {
        a.slE[oy + (size_t)i * Nz + k] = ey;
        a.slE[oy + (size_t)Nx * Nz + (size_t)i * Nz + k] = ez_slice;
    }
    if (i == a.ssx) {
        a.slE[ox + (size_t)j * Nz + k] = ey;
        a.slE[ox + (size_t)Ny * Nz + (size_t)j * Nz + k] = ez_slice;
    }
}
__device__ __forceinline__ void band_slices_h(const Args &a, int i, int j, int k, float hy, float hz) {
    const int Nx = a.Nx, Ny = a.Ny, Nz = a.Nz;
    const size_t oz = 0, oy = 2 * (size_t)Nx * Ny, ox = oy + 2 * (size_t)Nx * Nz;
    if (k == a.ssz && j < Ny - 1) {
        a.slH[oz + (size_t)i * Ny + j] = hy;
        a.slH[oz + (size_t)Nx * Ny + (size_t)i * Ny + j] = hz;
    }
    if (j == a.ssy && k < Nz - 1) {
        a.slH[oy + (size_t)i * Nz + k] = hy;
        a.slH[oy + (size_t)Nx * Nz + (size_t)i * Nz + k] = hz;
    }
    if (i == a.ssx && j < Ny - 1 && k < Nz - 1) {
        a.slH[ox + (size_t)j * Nz + k] = hy;
        a.slH[ox + (size_t)Ny * Nz + (size_t)j * Nz + k] = hz;
    }
}

// Values of a band cell loaded before its update (every load of the cell is
// then in flight at once; read where h_cell and e_cell use them, a load would
// wait behind the previous component's psi store, which may alias it).  A
// neighbour outside the grid reads as zero; the updates never use it.
struct PreSrc {
    float hv[3], ev[3], ej[3], ek[3], ei[3];
};
struct PreSrcView {
    const PreSrc &p;
    __device__ __forceinline__ float h(int c) const { return p.hv[c]; }
    __device__ __forceinline__ float e(int c) const { return p.ev[c]; }
    __device__ __forceinline__ float ej(int c) const { return p.ej[c]; }
    __device__ __forceinline__ float ek(int c) const { return p.ek[c]; }
    __device__ __forceinline__ float ei(int c) const { return p.ei[c]; }
};
struct PreHSrc {
    float hj[3], hk[3], hyi_, hzi_;
};
struct PreHSrcView {
    const PreHSrc &p;
    __device__ __forceinline__ float hj(int c) const { return p.hj[c]; }
    __device__ __forceinline__ float hk(int c) const { return p.hk[c]; }
    __device__ __forceinline__ float hyi() const { return p.hyi_; }
    __device__ __forceinline__ float hzi() const { return p.hzi_; }
};

template <int PAR>
__global__ void __launch_bounds__(256) k_fp32_band_h(const __grid_constant__ Args a, int record) {
    const size_t row = a.Nzp, plane = (size_t)a.Ny * a.Nzp;
    for_band_cells(a, [&](int i, int j, int k) {
        const size_t cg = (size_t)i * plane + (size_t)j * row + k;
        const float *const *E = a.E[PAR], *const *H = a.H[PAR];
        PreSrc ps;
        for (int c = 0; c < 3; c++) {
            ps.hv[c] = H[c][cg];
            ps.ev[c] = E[c][cg];
        }
        // neighbours the H update reads: Ez, Ex at +j; Ex, Ey at +k; Ey, Ez at +i
        const bool jn = j < a.Ny - 1, kn = k < a.Nz - 1, in = i < a.Nx - 1;
        ps.ej[1] = ps.ek[2] = ps.ei[0] = 0.f;
        ps.ej[0] = jn ? E[0][cg + row] : 0.f;
        ps.ej[2] = jn ? E[2][cg + row] : 0.f;
        ps.ek[0] = kn ? E[0][cg + 1] : 0.f;
        ps.ek[1] = kn ? E[1][cg + 1] : 0.f;
        ps.ei[1] = in ? E[1][cg + plane] : 0.f;
        ps.ei[2] = in ? E[2][cg + plane] : 0.f;
        const HVal hv = h_cell<PAR, false, true>(a, i, j, k, PreSrcView{ps}, true, true, true, false, a.dopml != 0);
        a.H[PAR ^ 1][0][cg] = hv.x;
        a.H[PAR ^ 1][1][cg] = hv.y;
        a.H[PAR ^ 1][2][cg] = hv.z;
        if (record) band_slices_h(a, i, j, k, hv.y, hv.z);
    });
}

// `xskip`: the pass (k_fp32_step_fast) did not march the band's x planes
// nor the tile rows wholly inside its y rows; their J is advanced here,
// before their E update, as the pass would.
template <int PAR, int JM>
__global__ void __launch_bounds__(256) k_fp32_band_e(const __grid_constant__ Args a, int record, int t, int xskip) {
    const size_t row = a.Nzp, plane = (size_t)a.Ny * a.Nzp;
    const int w = a.dopml ? a.L + 1 : 1;
    for_band_cells(a, [&](int i, int j, int k) {
        const size_t cg = (size_t)i * plane + (size_t)j * row + k;
        const float *const *Hn = a.H[PAR ^ 1];
        const HVal hv = {Hn[0][cg], Hn[1][cg], Hn[2][cg]};
        const float ex = a.E[PAR][0][cg], ey = a.E[PAR][1][cg], ez = a.E[PAR][2][cg];
        // neighbours the E update reads: new Hz, Hx at -j; Hy, Hx at -k; Hy, Hz at -i
        PreHSrc hs;
        hs.hj[1] = hs.hk[2] = 0.f;
        hs.hj[0] = j >= 1 ? Hn[0][cg - row] : 0.f;
        hs.hj[2] = j >= 1 ? Hn[2][cg - row] : 0.f;
        hs.hk[0] = k >= 1 ? Hn[0][cg - 1] : 0.f;
        hs.hk[1] = k >= 1 ? Hn[1][cg - 1] : 0.f;
        hs.hyi_ = i >= 1 ? Hn[1][cg - plane] : 0.f;
        hs.hzi_ = i >= 1 ? Hn[2][cg - plane] : 0.f;
        // J as the pass left it: advanced where the block holds plasma, zero
        // elsewhere (read only where the block holds plasma).
        float jx = 0.f, jy = 0.f, jz = 0.f;
        if (!a.plasma || a.plasma[(size_t)i * a.ntiles + (j / TJ) * a.ntk + k / TK]) {
            jx = a.J[0][cg];
            jy = a.J[1][cg];
            jz = a.J[2][cg];
            const int j0 = (j / TJ) * TJ;  // the cell's tile row (skipped by the fast pass when in the band)
            if (JM != 2 && xskip && (i < w || i >= a.Nx - w || j0 + TJ <= w || j0 >= a.Ny - w) && t > 0 &&
                i >= 1 && i < a.Nx - 1 && j >= 1 && j < a.Ny - 1 && k >= 1 && k < a.Nz - 1) {
                const size_t ij = (size_t)i * a.Ny + j;
                const float cwq = a.wq3 ? a.wq3[cg] : a.wq2[ij];
                const float cnu = JM == 0 ? (a.nu3 ? a.nu3[cg] : a.nu2[ij]) : 0.f;
                j_advance<JM>(a, a.lku, cwq, cnu, a.G[k], a.G2[k], ex, ey, ez, a.E[PAR][0][cg - plane],
                              a.E[PAR][1][cg - row], a.E[PAR][2][cg - 1], jx, jy, jz);
                a.J[0][cg] = jx;
                a.J[1][cg] = jy;
                a.J[2][cg] = jz;
            }
        }
        const EVal ev = e_cell<PAR, false, true>(a, i, j, k, ex, ey, ez, hv, PreHSrcView{hs}, jx, jy, jz, false,
                                                 a.dopml != 0);
        a.E[PAR ^ 1][0][cg] = ev.x;
        a.E[PAR ^ 1][1][cg] = ev.y;
        a.E[PAR ^ 1][2][cg] = ev.z;
        if (record) band_slices_e(a, i, j, k, ev.y, ev.z_slice);
    });
}

// Slices of the current state (set `cur`) in the record layout, E block
// (is_h = 0) or H block, optionally minus the incident field inside the
// total-field region.
__global__ void k_fp32_slices(const __grid_constant__ Args a, IncidentWave<float> w, int cur, int is_h,
                              int scattered, double *out, size_t n) {
    const size_t plane = (size_t)a.Ny * a.Nzp;
    for (size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (size_t)gridDim.x * blockDim.x) {
        SliceCell c;
        double v = 0.0;
        if (slice_cell_of(q, a.Nx, a.Ny, a.Nz, a.ssx, a.ssy, a.ssz, is_h != 0, &c)) {
            const size_t x = (size_t)c.i * plane + (size_t)c.j * a.Nzp + c.k;
            if (is_h) {
                v = (double)a.H[cur][1 + c.comp][x];
                if (scattered) v -= w.h(1 + c.comp, c.i, c.j, c.k);
            } else {
                v = (double)a.E[cur][1 + c.comp][x];
                if (scattered) v -= w.e(1 + c.comp, c.i, c.j, c.k);
            }
        }
        out[q] = v;
    }
}

// The plasma table (Args::plasma): one warp per (plane, tile) block, lane =
// k column (coalesced rows of the map).  A block counts as plasma when any
// cell has a nonzero E0 omega_p^2 and a nonzero z factor (a superset of the
// cells whose J can leave zero).
__global__ void k_plasma_blocks(const __grid_constant__ Args a, unsigned char *out) {
    const size_t n = (size_t)a.Nx * a.ntiles;
    const int lane = threadIdx.x & 31;
    const size_t w0 = ((size_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5,
                 dw = ((size_t)gridDim.x * blockDim.x) >> 5;
    for (size_t u = w0; u < n; u += dw) {
        const int q = (int)(u / a.ntiles), tile = (int)(u % a.ntiles);
        const int k = (tile % a.ntk) * TK + lane, j0 = (tile / a.ntk) * TJ;
        bool any = false;
        if (k < a.Nz && a.G2[k] != 0.f)
            for (int dj = 0; dj < TJ && j0 + dj < a.Ny; dj++) {
                const size_t ij = (size_t)q * a.Ny + j0 + dj;
                if ((a.wq3 ? a.wq3[ij * a.Nzp + k] : a.wq2[ij]) != 0.f) any = true;
            }
        any = __any_sync(0xffffffffu, any);
        if (lane == 0) out[u] = any ? 1 : 0;
    }
}

// E probes of the final step (the per-step ones ride in the next pass).
__global__ void k_fp32_flush(const Args a, int t_last, int par) {
    const int p = threadIdx.x;
    if (p >= a.nprobes) return;
    // `par`: the set written by the last pass
    const size_t sI = (size_t)a.Ny * a.Nzp, sJ = a.Nzp;
    const int ix = a.probe_ijk[3 * p], iy = a.probe_ijk[3 * p + 1], iz = a.probe_ijk[3 * p + 2];
    const size_t c = ix * sI + iy * sJ + iz;
    const float *E0 = a.E[par][0], *E1 = a.E[par][1], *E2 = a.E[par][2];
    const float *H0 = a.H[par][0], *H1 = a.H[par][1], *H2 = a.H[par][2];
    const size_t o = (size_t)t_last * a.nprobes + p, T = (size_t)a.tsteps * a.nprobes;
    a.probe[o] = 0.5 * ((double)E0[c] + E0[c - sI]);
    a.probe[T + o] = 0.5 * ((double)E1[c] + E1[c - sJ]);
    a.probe[2 * T + o] = 0.5 * ((double)E2[c] + E2[c - 1]);
    a.probe[3 * T + o] = 0.25 * ((double)H0[c] + H0[c - sJ] + H0[c - 1] + H0[c - sJ - 1]);
    a.probe[4 * T + o] = 0.25 * ((double)H1[c] + H1[c - sI] + H1[c - 1] + H1[c - sI - 1]);
    a.probe[5 * T + o] = 0.25 * ((double)H2[c] + H2[c - sJ] + H2[c - sI] + H2[c - sI - sJ]);
}

// max |Ex| (record steps) and the non-finite guard, over the padded grid.
__global__ void __launch_bounds__(256) k_fp32_scan(const float *__restrict__ ex,
                                                   const float *__restrict__ ey,
                                                   const float *__restrict__ ez, size_t n,
                                                   unsigned int *maxbits, unsigned int *bad) {
    float m = 0.f;
    unsigned int nb = 0;
    for (size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x; q < n;
         q += (size_t)gridDim.x * blockDim.x) {
        const float a = ex[q];
        const float v = fabsf(a);
        if (v > m) m = v;
        nb |= !isfinite(a) | !isfinite(ey[q]) | !isfinite(ez[q]);
    }
    for (int off = 16; off > 0; off >>= 1) {
        m = fmaxf(m, __shfl_down_sync(0xffffffffu, m, off));
        nb |= __shfl_down_sync(0xffffffffu, nb, off);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMax(maxbits, __float_as_uint(m));
        if (nb) atomicOr(bad, 1u);
    }
}

// E0 * omega_p^2 of a parametric trail in the padded [Nx][Ny][Nzp] layout.
__global__ void k_trail_wq(TrailDev t, int Nzp, float *out) {
    const size_t n = (size_t)t.Nx * t.Ny * Nzp;
    for (size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x; q < n;
         q += (size_t)gridDim.x * blockDim.x) {
        const int k = (int)(q % Nzp);
        const size_t ij = q / Nzp;
        out[q] = k < t.Nz ? trail_wq_f32(t, (int)(ij / t.Ny), (int)(ij % t.Ny), k) : 0.f;
    }
}

// Copy one slice/field buffer of floats to doubles.
__global__ void k_f2d(const float *__restrict__ in, double *__restrict__ out, size_t n) {
    for (size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x; q < n;
         q += (size_t)gridDim.x * blockDim.x)
        out[q] = in[q];
}

// Unpadded [Nx][Ny][Nz] view of a padded [Nx][Ny][Nzp] component.
__global__ void k_unpad(const float *__restrict__ in, double *__restrict__ out, int Nx, int Ny,
                        int Nz, int Nzp) {
    const size_t n = (size_t)Nx * Ny * Nz;
    for (size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x; q < n;
         q += (size_t)gridDim.x * blockDim.x) {
        const size_t k = q % Nz, ij = q / Nz;
        out[q] = in[ij * Nzp + k];
    }
}

using EncodeFn = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                              const cuuint64_t *, const cuuint32_t *, const cuuint32_t *,
                              CUtensorMapInterleave, CUtensorMapSwizzle, CUtensorMapL2promotion,
                              CUtensorMapFloatOOBfill);

EncodeFn encoder() {
    static EncodeFn fn = nullptr;
    if (!fn) {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess || !p)
            throw Error(MFDTD_ECUDA, "cuTensorMapEncodeTiled is not available");
        fn = (EncodeFn)p;
    }
    return fn;
}

// 4-D map of the six field components of one parity, [6][Nx][Ny][Nzp] floats
// (k fastest), read as boxes of bk x bj x 1 plane x 6 components.  Elements
// at k >= Nz or outside the grid read as zero.
void make_map(CUtensorMap *m, float *base, int Nx, int Ny, int Nz, int Nzp, int bk, int bj) {
    const cuuint64_t NC = (cuuint64_t)Nx * Ny * Nzp;
    cuuint64_t dims[4] = {(cuuint64_t)Nz, (cuuint64_t)Ny, (cuuint64_t)Nx, 6};
    cuuint64_t strides[3] = {(cuuint64_t)Nzp * 4, (cuuint64_t)Ny * Nzp * 4, NC * 4};
    cuuint32_t box[4] = {(cuuint32_t)bk, (cuuint32_t)bj, 1, 6};
    cuuint32_t es[4] = {1, 1, 1, 1};
    CUresult r = encoder()(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, base, dims, strides, box, es,
                           CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                           CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) throw Error(MFDTD_ECUDA, "cuTensorMapEncodeTiled failed: " + std::to_string((int)r));
}

void ck(cudaError_t e, const char *what) {
    if (e != cudaSuccess) throw Error(MFDTD_ECUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

}  // namespace

struct Fp32Sim::Impl {
    Args a;
    Args af;        // the fast pass's Args: the same, over the planes [L + 1, Nx - L - 1)
    dim3 grid_fast;
    Maps maps;
    Maps mapsw;     // boxes of the wide interior pass (8 x 64 tiles)
    std::vector<void *> allocs;
    int64_t bytes = 0;
    int Nx = 0, Ny = 0, Nz = 0, Nzp = 0, tsteps = 0, nntf = 0, nprobes = 0;
    size_t slice_len = 0;
    dim3 grid;
    double *dtmp = nullptr;      // FP64 staging for conversions
    size_t dtmp_len = 0;
    unsigned int *scan = nullptr;  // [0] max|Ex| bits, [1] bad flag
    int jm = 0;  // J method of the kernel variant
    int sms = 148;                 // SM count (grids of the follow-up kernels)
    double plasma_fraction = 1.0;  // share of (plane, tile) blocks holding plasma
    std::vector<int> tile_order;   // host copy: boundary tiles first
    int n_boundary = 0;            // how many of them are boundary tiles
    bool fast_ok = false;          // non-record passes may use k_fp32_step_fast
    long long n_fast = 0, n_general = 0;  // passes run by each pass kernel
    // Non-record passes as k_fp32_step_wide over the interior tiles and planes
    // plus k_fp32_slab over the rest, on a second stream (see k_fp32_slab);
    // else k_fp32_step_fast followed by the band kernels.
    bool slab_ok = false;
    const int4 *slab_items = nullptr;
    int n_slab_items = 0;
    // Running DFT (single simulations): the ring of face values (allocated at
    // the first step: batch members never use it), the FP32 phase table, and
    // the ring's first step and fill.
    float *ntf_ring = nullptr;
    const float4 *phase4 = nullptr;
    size_t nface = 0;
    int ring_t0 = 0, ring_fill = 0;
    // the Huygens faces and the nodes behind them lie outside the TF/SF band
    bool ntf_outside_band = false;
    cudaStream_t aux = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    cudaEvent_t ev_post = nullptr, ev_dft = nullptr;  // the DFT copy beside the TF/SF corrections
    // In a batch of class 1 (Fp32Sim::batch_class): the tiles whose cells are
    // all interior in j and k (fast path over the interior planes, slab march
    // over the x-slab planes) and the rest (slab march over every plane);
    // w = L + 1 with the CPML, else 1.
    bool slab_eligible = false;
    int wband = 1;
    std::vector<int> inner32, edge32;
    // The same members with 8 x 64 tiles: pairs of neighbouring interior
    // tiles (left tile ids) on the wide path, every other tile on the slab
    // march.
    std::vector<int> pairs32, edgew;


    // Device memory comes from the device's stream-ordered pool (see
    // configure_pool), zeroed on the simulation's stream.
    template <class T> T *alloc(size_t n, cudaStream_t s) {
        void *p = nullptr;
        size_t b = std::max<size_t>(n, 1) * sizeof(T);
        ck(cudaMallocAsync(&p, b, s), "cudaMallocAsync");
        allocs.push_back(p);
        bytes += (int64_t)b;
        // TMA and the 16-byte vector accesses want at least 256-byte alignment
        if (reinterpret_cast<uintptr_t>(p) % 256) throw Error(MFDTD_ECUDA, "pool allocation not 256-byte aligned");
        ck(cudaMemsetAsync(p, 0, b, s), "cudaMemset");
        return (T *)p;
    }
    template <class T> T *upload(const std::vector<T> &v, cudaStream_t s) {
        T *d = alloc<T>(v.size(), s);
        if (!v.empty()) ck(cudaMemcpyAsync(d, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, s), "H2D");
        return d;
    }
    ~Impl() {
        if (aux) {
            cudaStreamSynchronize(aux);
            cudaStreamDestroy(aux);
        }
        if (ev_fork) cudaEventDestroy(ev_fork);
        if (ev_join) cudaEventDestroy(ev_join);
        if (ev_post) cudaEventDestroy(ev_post);
        if (ev_dft) cudaEventDestroy(ev_dft);
        // No kernel may still use the memory when it goes back to the pool
        // (as cudaFree would ensure); the frees then take no unmapping.
        if (!allocs.empty()) cudaDeviceSynchronize();
        for (void *p : allocs) cudaFreeAsync(p, 0);
    }
};

int64_t Fp32Sim::footprint(const Problem &P) {
    const int64_t Nzp = (P.Nz + TK - 1) / TK * TK;
    const int64_t cells = (int64_t)P.Nx * P.Ny * Nzp;
    const int64_t L2 = 2 * P.L;
    const int64_t psi = P.dopml ? (L2 * P.Ny * P.Nz + (int64_t)P.Nx * L2 * P.Nz + (int64_t)P.Nx * P.Ny * L2) * 2 : 0;
    const int64_t nf2 = 2 * P.nntf();
    const int64_t ntf = 8 * nf2 * ((int64_t)P.Ny * P.Nz + (int64_t)P.Nx * P.Nz + (int64_t)P.Nx * P.Ny);
    const int64_t maps = cells * 4 * ((P.wp3.empty() && !P.has_trail ? 0 : 1) + (P.nu3.empty() ? 0 : 1));
    // band kernels' unit table (an upper bound) and the plasma-block table
    const int64_t w = P.dopml ? P.L + 1 : 1, nseg = (P.Nz + 31) / 32, nsegz = (2 * w + 31) / 32;
    const int64_t band = 8 * (2 * w * P.Ny * nseg + (int64_t)P.Nx * 2 * w * nseg + (int64_t)P.Nx * P.Ny * nsegz);
    const int64_t ntiles = (Nzp / TK) * ((P.Ny + TJ - 1) / TJ);
    const int64_t ptab = (int64_t)P.Nx * ntiles;
    const int64_t slab = 16 * ntiles * ((P.Nx + 95) / 96 + 2);  // slab-march items (an upper bound)
    // Lee-Kalluri table: a matrix pair per cell (padded layout) when nu varies
    // along all three axes
    const int64_t lkt = (P.doB0 && P.lk_mode == LK_PER_CELL) ? cells * 4 * kLkStride : 4 * (int64_t)P.lk.size();
    // running-DFT ring of a single simulation and the split phase table
    const int64_t ring = P.nntf() > 0 ? 4 * (kNtfRing * 6 * 2 * ((int64_t)P.Ny * P.Nz + (int64_t)P.Nx * P.Nz +
                                                                 (int64_t)P.Nx * P.Ny) + 2 * (int64_t)P.tsteps * nf2)
                                      : 0;
    return cells * 4 * 15 + maps + psi * 4 * 3 + 8 * ntf + 8 * (int64_t)P.tsteps * (nf2 + 6 * P.nprobes() + 2) + band +
           ptab + slab + lkt + ring;
}

// The FP32 form takes its device memory from the device's default
// stream-ordered pool, set once per device to keep up to a quarter of the
// device's memory cached after frees: a simulation created after another one
// ended (a server's next job, a sweep's next trail, a second run in the same
// process) reuses that memory without new mappings, and freeing one takes no
// unmapping.  Memory beyond that goes back to the system at the next
// synchronisation.
static void configure_pool() {
    static std::mutex mu;
    static std::vector<int> done;
    int dev = 0;
    ck(cudaGetDevice(&dev), "cudaGetDevice");
    std::lock_guard<std::mutex> lk(mu);
    if (std::find(done.begin(), done.end(), dev) != done.end()) return;
    cudaMemPool_t pool;
    ck(cudaDeviceGetDefaultMemPool(&pool, dev), "cudaDeviceGetDefaultMemPool");
    size_t free_b = 0, total_b = 0;
    ck(cudaMemGetInfo(&free_b, &total_b), "cudaMemGetInfo");
    uint64_t keep = total_b / 4;
    ck(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep), "cudaMemPoolSetAttribute");
    done.push_back(dev);
}

// The axes whose CPML slabs or domain faces a slab-march tile touches, its
// halo row and column included (slab_view): bit 0 y, bit 1 z.
static int slab_yz(const Fp32Sim::Impl &m, int tl) {
    const int w = m.wband, j0 = (tl / m.a.ntk) * TJ, k0 = (tl % m.a.ntk) * TK;
    const bool yin = j0 - 1 >= w && j0 + TJ - 1 <= m.Ny - w - 1;
    const bool zin = k0 - 1 >= w && k0 + TK - 1 <= m.Nz - w - 1;
    return (yin ? 0 : 1) | (zin ? 0 : 2);
}

void Fp32Sim::init(const Problem &P, void *stream) {
    cudaStream_t s = (cudaStream_t)stream;
    if (P.L > kMaxPml) throw Error(MFDTD_EINVAL, "CPML too thick");
    configure_pool();
    impl_ = new Impl();
    Impl &m = *impl_;
    Args &a = m.a;
    std::memset(&a, 0, sizeof a);
    m.Nx = P.Nx; m.Ny = P.Ny; m.Nz = P.Nz; m.Nzp = (P.Nz + TK - 1) / TK * TK;
    m.tsteps = P.tsteps; m.nntf = P.nntf(); m.nprobes = P.nprobes();
    if (m.nprobes > 24) throw Error(MFDTD_EINVAL, "FP32 form supports at most 24 probes");
    a.Nx = P.Nx; a.Ny = P.Ny; a.Nz = P.Nz; a.Nzp = m.Nzp; a.L = P.L;
    a.xshift = P.xshift; a.yshift = P.yshift; a.zshift = P.zshift;
    a.psi_py = 2u * P.L * P.Nz;
    a.psi_pz = (unsigned)P.Ny * 2u * P.L;
    a.psi_px = (unsigned)P.Ny * P.Nz;
    a.bx1 = P.bx1; a.bx2 = P.bx2; a.by1 = P.by1; a.by2 = P.by2; a.bz1 = P.bz1; a.bz2 = P.bz2;
    a.ntfb = P.ntfb; a.nntf = P.nntf(); a.ssx = P.ssx; a.ssy = P.ssy; a.ssz = P.ssz;
    a.dopml = P.dopml; a.doplate = P.doplate; a.doB0 = P.doB0; a.lk_mode = P.lk_mode;
    a.plate_lo = P.plate_lo; a.plate_up = P.plate_up; a.nprobes = P.nprobes(); a.tsteps = P.tsteps;
    a.c1h = (float)P.c1h; a.c2h = (float)P.c2h;
    a.chx = (float)(P.c2h / P.dx); a.chy = (float)(P.c2h / P.dy); a.chz = (float)(P.c2h / P.dz);
    a.c1e0 = (float)P.c1e0; a.c2e0 = (float)P.c2e0;
    a.cex = (float)(P.c2e0 / P.dx); a.cey = (float)(P.c2e0 / P.dy); a.cez = (float)(P.c2e0 / P.dz);
    a.c1s = (float)P.c1s; a.c2s = (float)P.c2s;
    a.csx = (float)(P.c2s / P.dx); a.csy = (float)(P.c2s / P.dy); a.csz = (float)(P.c2s / P.dz);
    a.dtf = (float)P.dt; a.c0di = (float)(2 * kE0 * P.dt);
    a.platesize = P.platesize;
    a.kappa_on = P.kappa_on;
    a.oblique = P.oblique;
    a.lk_colocated = P.ext.lk_colocated;
    // A single simulation runs the DFT and (without a plate or sphere, whose
    // per-cell coefficients the follow-up pass does not carry) the oblique
    // TF/SF corrections as kernels of their own after each pass.
    a.obl_inline = (P.oblique && P.doplate != 0) ? 1 : 0;
    // The CPML slabs and domain edges are recomputed by the band kernels
    // after each pass, where the grid has an interior on every axis.
    {
        const int w = P.dopml ? P.L + 1 : 1;
        a.band = (P.Nx > 2 * w && P.Ny > 2 * w && P.Nz > 2 * w && P.Nx < 65536 && P.Ny < 65536 && P.Nz < 65536)
                     ? 1 : 0;
        a.band_units = nullptr;
        a.n_band_units = 0;
        if (a.band) {  // the band kernels' work units (see for_band_cells)
            std::vector<int2> u;
            auto unit = [&](int i, int j, int m0, int n, int list) {
                u.push_back(make_int2((int)((unsigned)i | ((unsigned)j << 16)),
                                      m0 | (n << 16) | (list << 24)));
            };
            auto full_row = [&](int i, int j) {
                for (int k0 = 0; k0 < P.Nz; k0 += 32) unit(i, j, k0, std::min(32, P.Nz - k0), 0);
            };
            for (int p = 0; p < 2 * w; p++)
                for (int j = 0; j < P.Ny; j++) full_row(p < w ? p : P.Nx - 2 * w + p, j);
            for (int i = w; i < P.Nx - w; i++)
                for (int jb = 0; jb < 2 * w; jb++) full_row(i, jb < w ? jb : P.Ny - 2 * w + jb);
            for (int i = w; i < P.Nx - w; i++)
                for (int j = w; j < P.Ny - w; j++)
                    for (int m0 = 0; m0 < 2 * w; m0 += 32) unit(i, j, m0, std::min(32, 2 * w - m0), 1);
            a.band_units = m.upload(u, s);
            a.n_band_units = (int)u.size();
        }
    }
    Tables T;
    std::memset(&T, 0, sizeof T);
    if (P.oblique) {
        a.M = P.M; a.ashift = P.ashift; a.s0 = (float)P.s0;
        for (int q = 0; q < 3; q++) {
            a.kr[q] = (float)P.kr[q]; a.ke[q] = (float)P.inc_e[q]; a.kh[q] = (float)P.inc_h[q];
        }
        a.chl = (float)(P.c2h / P.dl); a.cel = (float)(P.c2e0 / P.dl);
        for (int q = 0; q < 2 * P.L; q++) {
            T.Bh1[q] = (float)P.Bh1[q]; T.Ah1[q] = (float)(P.Ah1[q] / P.dl);
            T.Be1[q] = (float)P.Be1[q]; T.Ae1[q] = (float)(P.Ae1[q] / P.dl);
        }
    }
    for (int q = 0; q < 2 * P.L; q++) {
        T.Khx[q] = (float)(P.Kh[q] / P.dx); T.Khy[q] = (float)(P.Kh[q] / P.dy); T.Khz[q] = (float)(P.Kh[q] / P.dz);
        T.Kex[q] = (float)(P.Ke[q] / P.dx); T.Key[q] = (float)(P.Ke[q] / P.dy); T.Kez[q] = (float)(P.Ke[q] / P.dz);
        T.Bh[q] = (float)P.Bh[q];
        T.Ahx[q] = (float)(P.Ah[q] / P.dx); T.Ahy[q] = (float)(P.Ah[q] / P.dy); T.Ahz[q] = (float)(P.Ah[q] / P.dz);
        T.Be[q] = (float)P.Be[q];
        T.Aex[q] = (float)(P.Ae[q] / P.dx); T.Aey[q] = (float)(P.Ae[q] / P.dy); T.Aez[q] = (float)(P.Ae[q] / P.dz);
    }
    {
        Tables *d = m.alloc<Tables>(1, s);
        ck(cudaMemcpyAsync(d, &T, sizeof T, cudaMemcpyHostToDevice, s), "H2D");
        a.tb = d;
    }
    const size_t NC = (size_t)P.Nx * P.Ny * m.Nzp;
    for (int b = 0; b < 2; b++) {  // one block per parity: Ex Ey Ez Hx Hy Hz (one TMA map)
        float *f = m.alloc<float>(6 * NC, s);
        for (int c = 0; c < 3; c++) {
            a.E[b][c] = f + c * NC;
            a.H[b][c] = f + (3 + c) * NC;
        }
    }
    for (int c = 0; c < 3; c++) a.J[c] = m.alloc<float>(NC, s);
    const size_t L2 = 2 * (size_t)P.L;
    const size_t nxs = L2 * P.Ny * P.Nz, nys = (size_t)P.Nx * L2 * P.Nz, nzs = (size_t)P.Nx * P.Ny * L2;
    const size_t psz[6] = {nys, nzs, nxs, nzs, nxs, nys};  // xy, xz, yx, yz, zx, zy
    if (P.dopml) {
        for (int q = 0; q < 6; q++) {
            a.Ph[0][q] = m.alloc<float>(psz[q], s);
            a.Ph[1][q] = m.alloc<float>(psz[q], s);
            a.Pe[q] = m.alloc<float>(psz[q], s);
        }
    }
    const size_t nline = std::max<size_t>(P.Nx, P.oblique ? (size_t)P.M : 0) + 1;
    for (int b = 0; b < 2; b++)
        for (int q = 0; q < 4; q++) {
            a.inc[b][q] = m.alloc<float>(nline, s);
            a.incP[b][q] = m.alloc<float>(L2, s);
        }
    {
        std::vector<float> wq2(P.wp2e.size()), nu2(P.nu2e.size()), G(P.Nz), G2(P.Nz);
        for (size_t q = 0; q < wq2.size(); q++) wq2[q] = (float)(kE0 * P.wp2e[q] * P.wp2e[q]);
        for (size_t q = 0; q < nu2.size(); q++) nu2[q] = (float)P.nu2e[q];
        // A per-cell map replaces the 2-D map times the z profile: its G factor is 1.
        const bool w3 = (!P.wp3.empty() || P.has_trail) && !P.doplate;
        const bool n3 = !P.nu3.empty() && !P.doplate;
        for (int k = 0; k < P.Nz; k++) {
            G[k] = n3 ? 1.f : (float)P.G[k];
            G2[k] = w3 ? 1.f : (float)(P.G[k] * P.G[k]);
        }
        auto per_cell = [&](const std::vector<double> &v, bool square) {
            std::vector<float> out((size_t)P.Nx * P.Ny * m.Nzp, 0.f);
            for (size_t ij = 0; ij < (size_t)P.Nx * P.Ny; ij++)
                for (int k = 0; k < P.Nz; k++) {
                    const double x = v[ij * P.Nz + k];
                    out[ij * m.Nzp + k] = (float)(square ? kE0 * x * x : x);
                }
            return out;
        };
        if (w3 && P.has_trail) {  // generated on the device: no per-cell host array
            float *wq = m.alloc<float>((size_t)P.Nx * P.Ny * m.Nzp, s);
            k_trail_wq<<<152 * 8, 256, 0, s>>>(trail_dev(P), m.Nzp, wq);
            ck(cudaGetLastError(), "trail map");
            a.wq3 = wq;
        } else {
            a.wq3 = w3 ? m.upload(per_cell(P.wp3, true), s) : nullptr;
        }
        a.nu3 = n3 ? m.upload(per_cell(P.nu3, false), s) : nullptr;
        a.wq2 = m.upload(wq2, s); a.nu2 = m.upload(nu2, s); a.G = m.upload(G, s); a.G2 = m.upload(G2, s);
        // Lee-Kalluri matrices (18 per entry): per k, per (i,j), or per cell.
        // A per-cell table is stored in the padded field layout, so the
        // kernels index it by the cell's offset (source/meteor-fork.cpp:1546-1573
        // builds one matrix pair per cell when nu varies along all three axes).
        std::vector<float> lk;
        if (P.lk_mode == LK_PER_CELL && !P.lk.empty()) {
            lk.assign((size_t)P.Nx * P.Ny * m.Nzp * kLkStride, 0.f);
            for (size_t ij = 0; ij < (size_t)P.Nx * P.Ny; ij++)
                for (int k = 0; k < P.Nz; k++)
                    for (int u = 0; u < kLkStride; u++)
                        lk[(ij * m.Nzp + k) * kLkStride + u] = (float)P.lk[(ij * P.Nz + k) * kLkStride + u];
        } else {
            lk.assign(P.lk.begin(), P.lk.end());
        }
        a.lk = m.upload(lk, s);
        std::vector<float> src(P.src.begin(), P.src.end());
        a.src = m.upload(src, s);
    }
    if (P.nntf() > 0) {
        m.nface = 2 * ((size_t)P.Ny * P.Nz + (size_t)P.Nx * P.Nz + (size_t)P.Nx * P.Ny);
        const int nb = P.ntfb;
        m.ntf_outside_band = nb >= 1 && nb + 2 <= std::min(P.bx1, std::min(P.by1, P.bz1)) && P.Nx - nb >= P.bx2 + 2 &&
                             P.Ny - nb >= P.by2 + 2 && P.Nz - nb >= P.bz2 + 2;
        // per (step, frequency): the phase's FP32 high parts and remainders
        std::vector<float4> pf(P.phase.size() / 2);
        for (size_t q = 0; q < pf.size(); q++) {
            const double c = P.phase[2 * q], sn = P.phase[2 * q + 1];
            const float ch = (float)c, sh = (float)sn;
            pf[q] = make_float4(ch, sh, (float)(c - (double)ch), (float)(sn - (double)sh));
        }
        m.phase4 = m.upload(pf, s);
        a.phase4 = m.phase4;
    }
    a.xc = m.upload(P.x, s); a.yc = m.upload(P.y, s); a.zc = m.upload(P.z, s);
    const size_t nf2 = 2 * (size_t)P.nntf();
    const size_t fb = (size_t)P.Ny * P.Nz * nf2, tb = (size_t)P.Nx * P.Nz * nf2, lr = (size_t)P.Nx * P.Ny * nf2;
    for (int q = 0; q < 24; q++) a.ntf[q] = m.alloc<double>(q < 8 ? fb : q < 16 ? tb : lr, s);
    a.probe = m.alloc<double>((size_t)6 * P.tsteps * P.nprobes(), s);
    std::vector<int> ijk;
    for (int n = 0; n < P.nprobes(); n++) { ijk.push_back(P.probex[n]); ijk.push_back(P.probey[n]); ijk.push_back(P.probez[n]); }
    a.probe_ijk = m.upload(ijk, s);
    m.slice_len = 2 * ((size_t)P.Nx * P.Ny + (size_t)P.Nx * P.Nz + (size_t)P.Ny * P.Nz);
    a.slE = m.alloc<float>(m.slice_len, s);
    a.slH = m.alloc<float>(m.slice_len, s);
    a.err = m.alloc<unsigned int>(1, s);
    m.scan = m.alloc<unsigned int>(2, s);
    m.dtmp_len = std::max(m.slice_len, (size_t)1);
    m.dtmp = m.alloc<double>(m.dtmp_len, s);

    for (int b = 0; b < 2; b++) {
        make_map(&m.maps.F[b], a.E[b][0], P.Nx, P.Ny, P.Nz, m.Nzp, EK, EJ);
        make_map(&m.mapsw.F[b], a.E[b][0], P.Nx, P.Ny, P.Nz, m.Nzp, EKW, EJ);
    }

    {
        auto attr = [](const void *f) {
            ck(cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_B), "attr");
        };
        attr((const void *)k_fp32_step<0, 0>); attr((const void *)k_fp32_step<1, 0>);
        attr((const void *)k_fp32_step<0, 1>); attr((const void *)k_fp32_step<1, 1>);
        attr((const void *)k_fp32_step<0, 2>); attr((const void *)k_fp32_step<1, 2>);
        // Four CTAs of the fast pass need 226 KB of shared memory: ask for the
        // largest carve-out.
        auto attr4 = [&](const void *f) {
            attr(f);
            ck(cudaFuncSetAttribute(f, cudaFuncAttributePreferredSharedMemoryCarveout, 100), "attr");
        };
        attr4((const void *)k_fp32_step_fast<0, 0>); attr4((const void *)k_fp32_step_fast<1, 0>);
        attr4((const void *)k_fp32_step_fast<0, 1>); attr4((const void *)k_fp32_step_fast<1, 1>);
        auto attrs = [&](const void *f, int bytes) {
            ck(cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes), "attr");
            ck(cudaFuncSetAttribute(f, cudaFuncAttributePreferredSharedMemoryCarveout, 100), "attr");
        };
        attrs((const void *)k_fp32_slab<0, 0>, SMEM_BS); attrs((const void *)k_fp32_slab<1, 0>, SMEM_BS);
        attrs((const void *)k_fp32_slab<0, 1>, SMEM_BS); attrs((const void *)k_fp32_slab<1, 1>, SMEM_BS);
        attrs((const void *)k_fp32_step_wide<0, 0>, SMEM_BW); attrs((const void *)k_fp32_step_wide<1, 0>, SMEM_BW);
        attrs((const void *)k_fp32_step_wide<0, 1>, SMEM_BW); attrs((const void *)k_fp32_step_wide<1, 1>, SMEM_BW);
    }
    m.jm = 0;
    if (P.doB0) {
        bool uniform = !P.lk.empty();
        for (size_t q = 18; q < P.lk.size() && uniform; q++) uniform = P.lk[q] == P.lk[q % 18];
        m.jm = uniform ? 1 : 2;
        if (uniform)
            for (int q = 0; q < 18; q++) a.lku[q] = (float)P.lk[q];
    }
    // Split x into chunks: enough work items to fill the machine several
    // times over on small grids, and on long x extents chunks of about 160
    // planes, so that the slower boundary tiles come as short items at the
    // head of each chunk round rather than as full-length marches that all
    // run side by side (768x768x1536: 16.44 ms per step in one chunk, 15.48
    // in 4 to 6, 15.74 in 16 -- each chunk re-computes one warm-up plane).
    int dev = 0, sms = 148;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    m.sms = sms;
    const int tiles = (m.Nzp / TK) * ((P.Ny + TJ - 1) / TJ);
    const int want = sms * 2 * 8;
    int chunks = std::max(1, std::min(P.Nx / 16 > 0 ? P.Nx / 16 : 1, (want + tiles - 1) / tiles));
    chunks = std::max(chunks, (P.Nx + 159) / 160);
    a.chunk = (P.Nx + chunks - 1) / chunks;
    chunks = (P.Nx + a.chunk - 1) / a.chunk;
    m.grid = dim3(tiles, 1, chunks);
    a.xbeg = 0;
    a.xend = P.Nx;
    {
        // Same test as the device's tile classification on non-record steps.
        const int ntk = m.Nzp / TK, nty = (P.Ny + TJ - 1) / TJ;
        const int Lc = P.dopml ? P.L : 0;
        auto hits = [](int lo, int hi, int v) { return v >= lo && v <= hi; };
        std::vector<int> order, later;
        for (int ty = 0; ty < nty; ty++)
            for (int tk = 0; tk < ntk; tk++) {
                const int jlo = ty * TJ - 1, jhi = ty * TJ + TJ, klo = tk * TK - 1, khi = tk * TK + TK;
                bool cl = P.doplate == 0;
                if (!a.band)
                    cl = cl && jlo >= Lc + 1 && jhi <= P.Ny - Lc - 2 && klo >= Lc + 1 && khi <= P.Nz - Lc - 2 &&
                         jlo >= 1 && jhi <= P.Ny - 2 && klo >= 1 && khi <= P.Nz - 2;
                const int sy[6] = {P.by1 - 1, P.by1, P.by2 - 1, P.by2, P.ntfb, P.Ny - P.ntfb};
                const int sz[6] = {P.bz1 - 1, P.bz1, P.bz2 - 1, P.bz2, P.ntfb, P.Nz - P.ntfb};
                const int q0 = (a.oblique && !a.obl_inline) ? 4 : 0, q1 = 4;
                for (int q = q0; q < q1; q++) cl = cl && !hits(jlo, jhi, sy[q]) && !hits(klo, khi, sz[q]);
                (cl ? later : order).push_back(ty * ntk + tk);
            }
        m.n_boundary = (int)order.size();
        // Every tile clean and every plane interior on non-record steps: the
        // fast pass applies (k_fp32_step_fast; not with the per-k or per-cell
        // Lee-Kalluri table, whose 18 coefficients do not fit its registers).
        m.fast_ok = a.band && a.oblique && !a.obl_inline && P.doplate == 0 && m.jm != 2 &&
                    m.n_boundary == 0;
        order.insert(order.end(), later.begin(), later.end());
        m.tile_order = order;
        a.tile_order = m.upload(order, s);
        a.ntk = ntk;
        a.ntiles = ntk * nty;
    }
    {
        // Which (plane, tile) blocks hold plasma; the pass skips J elsewhere.
        const size_t nb = (size_t)P.Nx * a.ntiles;
        unsigned char *d = m.alloc<unsigned char>(nb, s);
        k_plasma_blocks<<<m.sms * 8, 256, 0, s>>>(a, d);
        ck(cudaGetLastError(), "plasma blocks");
        std::vector<unsigned char> h(nb);
        ck(cudaMemcpyAsync(h.data(), d, nb, cudaMemcpyDeviceToHost, s), "D2H");
        ck(cudaStreamSynchronize(s), "plasma blocks");
        size_t np = 0;
        for (unsigned char v : h) np += v;
        m.plasma_fraction = nb ? (double)np / (double)nb : 0.0;
        a.plasma = d;
    }
    {
        const int w = P.dopml ? P.L + 1 : 1;
        m.wband = w;
        m.slab_eligible = batch_class(P) == 1;
        if (m.slab_eligible) {
            for (int tl : m.tile_order) {
                const int j0 = (tl / a.ntk) * TJ, k0 = (tl % a.ntk) * TK;
                const bool in = j0 >= w && j0 + TJ <= P.Ny - w && k0 >= w && k0 + TK <= P.Nz - w;
                (in ? m.inner32 : m.edge32).push_back(tl);
            }
            if (m.inner32.empty()) m.slab_eligible = false;
            std::vector<char> is_in((size_t)a.ntiles, 0);
            for (int tl : m.inner32) is_in[tl] = 1;
            std::vector<char> paired((size_t)a.ntiles, 0);
            for (int ty = 0; ty * TJ < P.Ny; ty++)
                for (int tk = 0; tk + 1 < a.ntk; tk++) {
                    const int tl = ty * a.ntk + tk;
                    if (is_in[tl] && is_in[tl + 1]) {
                        m.pairs32.push_back(tl);
                        paired[tl] = paired[tl + 1] = 1;
                        tk++;
                    }
                }
            for (int tl : m.tile_order)
                if (!paired[tl]) m.edgew.push_back(tl);
        }
    }
    if (m.fast_ok) {
        // With the slab march: the wide interior pass marches pairs of tiles
        // whose cells are all interior in j and k, over the planes
        // [w, Nx - w); k_fp32_slab the rest.  Without it: the fast pass leaves
        // the band's x planes, and the tile rows lying wholly in the band's y
        // rows, to the band kernels.
        const int w = P.dopml ? P.L + 1 : 1, len = P.Nx - 2 * w;
        auto interior = [&](int tl) {
            const int j0 = (tl / a.ntk) * TJ, k0 = (tl % a.ntk) * TK;
            return j0 >= w && j0 + TJ <= P.Ny - w && k0 >= w && k0 + TK <= P.Nz - w;
        };
        std::vector<int> inner, edge;
        for (int tl : m.tile_order) (interior(tl) ? inner : edge).push_back(tl);
        // Pairs of neighbouring interior tiles (8 x 64 columns); a tile left
        // without a partner joins the slab march.
        std::vector<int> pairs;
        {
            std::vector<char> is_in((size_t)a.ntiles, 0);
            for (int tl : inner) is_in[tl] = 1;
            std::vector<int> rest;
            for (int ty = 0; ty * TJ < P.Ny; ty++)
                for (int tk = 0; tk < a.ntk; tk++) {
                    const int tl = ty * a.ntk + tk;
                    if (!is_in[tl]) continue;
                    if (tk + 1 < a.ntk && is_in[tl + 1]) {
                        pairs.push_back(tl);
                        tk++;
                    } else {
                        rest.push_back(tl);
                    }
                }
            for (int tl : rest) edge.push_back(tl);
            inner.clear();
            for (int tl : pairs) { inner.push_back(tl); inner.push_back(tl + 1); }
        }
        m.slab_ok = !pairs.empty() && len > 0;
        if (m.slab_ok) {
            std::vector<int4> items;
            // Tiles reaching into the y/z slabs: every plane, in x-chunks of
            // about 96 planes (long marches first).
            const int ce = std::max(1, (P.Nx + 95) / 96), cl = (P.Nx + ce - 1) / ce;
            for (int tl : edge)
                for (int ib = 0; ib < P.Nx; ib += cl)
                    items.push_back(make_int4(tl, ib, std::min(P.Nx, ib + cl), slab_yz(m, tl)));
            m.slab_items = m.upload(items, s);
            m.n_slab_items = (int)items.size();
        } else {
            inner.clear();
            for (int tl : m.tile_order) {
                const int j0 = (tl / a.ntk) * TJ;
                if (!(j0 + TJ <= w || j0 >= P.Ny - w)) inner.push_back(tl);
            }
        }
        // The wide pass marches its tile pairs over every plane (the x-slab
        // planes with their x-normal CPML terms); the fast pass the planes
        // [w, Nx - w).
        const int xb = m.slab_ok ? 0 : w, xl = m.slab_ok ? P.Nx : len;
        m.af = a;
        m.af.xbeg = xb;
        m.af.xend = xb + xl;
        const std::vector<int> &fast_tiles = m.slab_ok ? pairs : inner;
        m.af.tile_order = m.upload(fast_tiles, s);
        const int tf = std::max(1, (int)fast_tiles.size());
        int cf = std::max(1, std::min(xl / 16 > 0 ? xl / 16 : 1, (want + tf - 1) / tf));
        cf = std::max(cf, (xl + 159) / 160);
        m.af.chunk = (xl + cf - 1) / cf;
        cf = (xl + m.af.chunk - 1) / m.af.chunk;
        m.grid_fast = dim3((unsigned)fast_tiles.size(), 1, cf);
    }
    // The second stream, for the slab march.  (Running the DFT there, beside
    // the next step's pass, which only reads the state the DFT reads, was
    // measured: no gain, both are bound by DRAM bandwidth.)
    if (m.slab_ok) {
        ck(cudaStreamCreateWithFlags(&m.aux, cudaStreamNonBlocking), "cudaStreamCreate");
        ck(cudaEventCreateWithFlags(&m.ev_fork, cudaEventDisableTiming), "cudaEventCreate");
        ck(cudaEventCreateWithFlags(&m.ev_join, cudaEventDisableTiming), "cudaEventCreate");
        ck(cudaEventCreateWithFlags(&m.ev_post, cudaEventDisableTiming), "cudaEventCreate");
        ck(cudaEventCreateWithFlags(&m.ev_dft, cudaEventDisableTiming), "cudaEventCreate");
    }
    bytes_ = m.bytes;
}

double Fp32Sim::plasma_fraction() const { return impl_->plasma_fraction; }

int Fp32Sim::batch_class(const Problem &P) {
    const int w = P.dopml ? P.L + 1 : 1;
    const bool band = P.Nx > 2 * w && P.Ny > 2 * w && P.Nz > 2 * w && P.Nx < 65536 && P.Ny < 65536 && P.Nz < 65536;
    int jm = 0;
    if (P.doB0) {
        bool uniform = !P.lk.empty();
        for (size_t q = 18; q < P.lk.size() && uniform; q++) uniform = P.lk[q] == P.lk[q % 18];
        jm = uniform ? 1 : 2;
    }
    // the oblique TF/SF corrections run after the pass exactly when there is
    // no plate or sphere (see init)
    if (!(band && P.oblique && P.doplate == 0 && jm != 2)) return 0;
    bool jin = false, kin = false;  // some 8 x 32 tile interior in j and in k
    for (int j0 = 0; j0 < P.Ny && !jin; j0 += TJ) jin = j0 >= w && j0 + TJ <= P.Ny - w;
    for (int k0 = 0; k0 < P.Nz && !kin; k0 += TK) kin = k0 >= w && k0 + TK <= P.Nz - w;
    return jin && kin ? 1 : 0;
}

int Fp32Sim::kernel_classes() { return 3; }
long long Fp32Sim::fast_passes() const { return impl_->n_fast; }
long long Fp32Sim::general_passes() const { return impl_->n_general; }
const char *Fp32Sim::fast_pass_name() const {
    return impl_->slab_ok ? "k_fp32_step_wide+k_fp32_slab" : "k_fp32_step_fast";
}
int Fp32Sim::current_update() const { return impl_->jm; }
const char *Fp32Sim::kernel_name(int which) {
    return which == 0 ? "k_fp32_step" : which == 1 ? "k_fp32_tfsf" : "k_fp32_ntf";
}

int Fp32Sim::step(int t, bool record, void *stream, void *const *ev) {
    cudaStream_t s = (cudaStream_t)stream;
    Impl &m = *impl_;
    if (ev) cudaEventRecord((cudaEvent_t)ev[0], s);
    const int rec = record ? 1 : 0;
    auto go = [&](auto kern) { kern<<<m.grid, NTHREADS, SMEM_B, s>>>(m.maps, m.a, t, rec); };
    auto go_fast = [&](auto kern) { kern<<<m.grid_fast, NTHREADS, SMEM_B, s>>>(m.maps, m.af, t); };
    // The pass reads the set holding the current state and writes the other.
    const bool fast = m.fast_ok && !record;
    (fast ? m.n_fast : m.n_general) += 1;
    int launches = 1;
    if (fast && m.slab_ok) {
        // the slab march on the second stream, concurrently with the pass
        ck(cudaEventRecord(m.ev_fork, s), "cudaEventRecord");
        ck(cudaStreamWaitEvent(m.aux, m.ev_fork, 0), "cudaStreamWaitEvent");
        const dim3 g((unsigned)m.n_slab_items);
        if (m_cur_ == 0) {
            if (m.jm == 0) k_fp32_slab<0, 0><<<g, NTHREADS, SMEM_BS, m.aux>>>(m.maps, m.a, t, m.slab_items);
            else k_fp32_slab<0, 1><<<g, NTHREADS, SMEM_BS, m.aux>>>(m.maps, m.a, t, m.slab_items);
        } else {
            if (m.jm == 0) k_fp32_slab<1, 0><<<g, NTHREADS, SMEM_BS, m.aux>>>(m.maps, m.a, t, m.slab_items);
            else k_fp32_slab<1, 1><<<g, NTHREADS, SMEM_BS, m.aux>>>(m.maps, m.a, t, m.slab_items);
        }
        launches++;
    }
    auto go_wide = [&](auto kern) { kern<<<m.grid_fast, NTHREADS, SMEM_BW, s>>>(m.mapsw, m.af, t); };
    if (fast && m.slab_ok) {
        if (m_cur_ == 0) {
            if (m.jm == 0) go_wide(k_fp32_step_wide<0, 0>);
            else go_wide(k_fp32_step_wide<0, 1>);
        } else {
            if (m.jm == 0) go_wide(k_fp32_step_wide<1, 0>);
            else go_wide(k_fp32_step_wide<1, 1>);
        }
    } else if (fast) {
        if (m_cur_ == 0) {
            if (m.jm == 0) go_fast(k_fp32_step_fast<0, 0>);
            else go_fast(k_fp32_step_fast<0, 1>);
        } else {
            if (m.jm == 0) go_fast(k_fp32_step_fast<1, 0>);
            else go_fast(k_fp32_step_fast<1, 1>);
        }
    } else if (m_cur_ == 0) {
        if (m.jm == 0) go(k_fp32_step<0, 0>);
        else if (m.jm == 1) go(k_fp32_step<0, 1>);
        else go(k_fp32_step<0, 2>);
    } else {
        if (m.jm == 0) go(k_fp32_step<1, 0>);
        else if (m.jm == 1) go(k_fp32_step<1, 1>);
        else go(k_fp32_step<1, 2>);
    }
    if (fast && m.slab_ok) {
        ck(cudaEventRecord(m.ev_join, m.aux), "cudaEventRecord");
        ck(cudaStreamWaitEvent(s, m.ev_join, 0), "cudaStreamWaitEvent");
    } else if (m.a.band) {
        const int g = m.sms * 8, xs = fast ? 1 : 0;
        auto band_e = [&](auto kern) { kern<<<g, 256, 0, s>>>(m.a, rec, t, xs); };
        if (m_cur_ == 0) {
            k_fp32_band_h<0><<<g, 256, 0, s>>>(m.a, rec);
            if (m.jm == 0) band_e(k_fp32_band_e<0, 0>);
            else if (m.jm == 1) band_e(k_fp32_band_e<0, 1>);
            else band_e(k_fp32_band_e<0, 2>);
        } else {
            k_fp32_band_h<1><<<g, 256, 0, s>>>(m.a, rec);
            if (m.jm == 0) band_e(k_fp32_band_e<1, 0>);
            else if (m.jm == 1) band_e(k_fp32_band_e<1, 1>);
            else band_e(k_fp32_band_e<1, 2>);
        }
        launches += 2;
    }
    if (ev) cudaEventRecord((cudaEvent_t)ev[1], s);
    // The DFT copy reads only the Huygens-face cells, which the TF/SF
    // corrections do not touch (the faces lie outside the band): with the
    // second stream it runs beside them, and the step ends when both have.
    const bool tfsf = m.a.oblique && !m.a.obl_inline;
    const bool dft = m.a.nntf > 0;
    const bool dft_beside = dft && tfsf && m.aux && m.ntf_outside_band;
    if (dft) {
        if (!m.ntf_ring) {
            m.ntf_ring = m.alloc<float>((size_t)kNtfRing * 6 * m.nface, s);
            bytes_ = m.bytes;
        }
        if (m.ring_fill == 0) m.ring_t0 = t;
    }
    if (dft_beside) {
        ck(cudaEventRecord(m.ev_post, s), "cudaEventRecord");
        ck(cudaStreamWaitEvent(m.aux, m.ev_post, 0), "cudaStreamWaitEvent");
        k_fp32_ntf<<<m.sms * 8, 256, 0, m.aux>>>(m.a, m_cur_ ^ 1, m.ntf_ring, m.ring_fill);
        launches++;
        if (++m.ring_fill == kNtfRing) launches += drain_ntf(m.aux);
    }
    if (tfsf) {
        if (m_cur_ == 0) k_fp32_tfsf<0><<<m.sms * 8, 256, 0, s>>>(m.a, rec);
        else k_fp32_tfsf<1><<<m.sms * 8, 256, 0, s>>>(m.a, rec);
        launches++;
    }
    if (ev) cudaEventRecord((cudaEvent_t)ev[2], s);
    if (dft_beside) {
        ck(cudaEventRecord(m.ev_dft, m.aux), "cudaEventRecord");
        ck(cudaStreamWaitEvent(s, m.ev_dft, 0), "cudaStreamWaitEvent");
    } else if (dft) {
        k_fp32_ntf<<<m.sms * 8, 256, 0, s>>>(m.a, m_cur_ ^ 1, m.ntf_ring, m.ring_fill);
        launches++;
        if (++m.ring_fill == kNtfRing) launches += drain_ntf(stream);
    }
    if (ev) cudaEventRecord((cudaEvent_t)ev[3], s);
    m_cur_ ^= 1;
    return launches;
}

int Fp32Sim::drain_ntf(void *stream) {
    Impl &m = *impl_;
    if (m.ring_fill == 0) return 0;
    k_fp32_ntf_flush<<<m.sms * 8, 256, 0, (cudaStream_t)stream>>>(m.a, m.ntf_ring, m.phase4, m.ring_t0, m.ring_fill);
    m.ring_fill = 0;
    return 1;
}

void Fp32Sim::check(void *stream) {
    unsigned int err = 0;
    ck(cudaMemcpyAsync(&err, impl_->a.err, 4, cudaMemcpyDeviceToHost, (cudaStream_t)stream), "D2H");
    ck(cudaStreamSynchronize((cudaStream_t)stream), "sync");
    if (err) throw Error(MFDTD_ETIMEOUT, "FP32 step: a TMA wait ran out (device error flag set)");
}

void Fp32Sim::record_stage(double *dE, double *dH, unsigned int *bits, void *stream) {
    cudaStream_t s = (cudaStream_t)stream;
    Impl &m = *impl_;
    const size_t n = m.slice_len, Nx = m.Nx;
    // The caller invokes this right after the step's pass: the state is in
    // the set that pass wrote.
    const int cur = m_cur_;
    ck(cudaMemsetAsync(m.scan, 0, 8, s), "memset");
    const size_t NC = (size_t)m.Nx * m.Ny * m.Nzp;
    k_fp32_scan<<<m.sms * 8, 256, 0, s>>>(m.a.E[cur][0], m.a.E[cur][1], m.a.E[cur][2], NC, m.scan, m.scan + 1);
    ck(cudaMemcpyAsync(bits, m.scan, 8, cudaMemcpyDeviceToDevice, s), "D2D");
    k_f2d<<<256, 256, 0, s>>>(m.a.slE, dE, n);
    k_f2d<<<8, 256, 0, s>>>(m.a.inc[cur][0], dE + n, Nx);
    k_f2d<<<8, 256, 0, s>>>(m.a.inc[cur][1], dE + n + Nx, Nx);
    k_f2d<<<256, 256, 0, s>>>(m.a.slH, dH, n);
    k_f2d<<<8, 256, 0, s>>>(m.a.inc[cur][2], dH + n, Nx);
    k_f2d<<<8, 256, 0, s>>>(m.a.inc[cur][3], dH + n + Nx, Nx);
}

double Fp32Sim::guard(void *stream) {
    cudaStream_t s = (cudaStream_t)stream;
    Impl &m = *impl_;
    ck(cudaMemsetAsync(m.scan, 0, 8, s), "memset");
    const size_t NC = (size_t)m.Nx * m.Ny * m.Nzp;
    const int cur = m_cur_;
    k_fp32_scan<<<152 * 8, 256, 0, s>>>(m.a.E[cur][0], m.a.E[cur][1], m.a.E[cur][2], NC, m.scan, m.scan + 1);
    unsigned int bits[2];
    ck(cudaMemcpyAsync(bits, m.scan, 8, cudaMemcpyDeviceToHost, s), "D2H");
    ck(cudaStreamSynchronize(s), "sync");
    check(stream);
    return bits[1] ? 1.0 : 0.0;
}

void Fp32Sim::flush(int t_last, void *stream) {
    Impl &m = *impl_;
    if (m.nprobes <= 0) return;
    k_fp32_flush<<<1, 32, 0, (cudaStream_t)stream>>>(m.a, t_last, m_cur_);
}

void Fp32Sim::read_ntf(int q, double *out, void *stream) {
    Impl &m = *impl_;
    const size_t nf2 = 2 * (size_t)m.nntf;
    const size_t n = q < 8 ? (size_t)m.Ny * m.Nz * nf2 : q < 16 ? (size_t)m.Nx * m.Nz * nf2 : (size_t)m.Nx * m.Ny * nf2;
    ck(cudaMemcpyAsync(out, m.a.ntf[q], n * 8, cudaMemcpyDeviceToHost, (cudaStream_t)stream), "D2H");
}

void Fp32Sim::read_slices(int scattered, double *E, double *H, const double kr[3], double s0,
                          const double ke[3], const double kh[3], void *stream) {
    cudaStream_t s = (cudaStream_t)stream;
    Impl &m = *impl_;
    const int cur = m_cur_;
    const Args &a = m.a;
    IncidentWave<float> w{};
    w.oblique = a.oblique;
    w.b1[0] = a.bx1; w.b1[1] = a.by1; w.b1[2] = a.bz1;
    w.b2[0] = a.bx2; w.b2[1] = a.by2; w.b2[2] = a.bz2;
    w.ey = a.inc[cur][0]; w.ez = a.inc[cur][1]; w.hy = a.inc[cur][2]; w.hz = a.inc[cur][3];
    w.eline = a.inc[cur][1]; w.hline = a.inc[cur][2];  // the auxiliary line's E and H (oblique)
    for (int d = 0; d < 3; d++) { w.kr[d] = kr[d]; w.ke[d] = ke[d]; w.kh[d] = kh[d]; }
    w.s0 = s0;
    const size_t n = m.slice_len;
    k_fp32_slices<<<m.sms * 4, 256, 0, s>>>(m.a, w, cur, 0, scattered, m.dtmp, n);
    ck(cudaMemcpyAsync(E, m.dtmp, n * 8, cudaMemcpyDeviceToHost, s), "D2H");
    ck(cudaStreamSynchronize(s), "sync");
    k_fp32_slices<<<m.sms * 4, 256, 0, s>>>(m.a, w, cur, 1, scattered, m.dtmp, n);
    ck(cudaMemcpyAsync(H, m.dtmp, n * 8, cudaMemcpyDeviceToHost, s), "D2H");
    ck(cudaStreamSynchronize(s), "sync");
}

void Fp32Sim::read_probes(double *out, void *stream) {
    Impl &m = *impl_;
    size_t n = (size_t)6 * m.tsteps * m.nprobes;
    if (n) ck(cudaMemcpyAsync(out, m.a.probe, n * 8, cudaMemcpyDeviceToHost, (cudaStream_t)stream), "D2H");
}

void Fp32Sim::read_field(int comp, double *out, void *stream) {
    cudaStream_t s = (cudaStream_t)stream;
    Impl &m = *impl_;
    const int cur = m_cur_;
    const float *src = comp < 3 ? m.a.E[cur][comp] : comp < 6 ? m.a.H[cur][comp - 3] : m.a.J[comp - 6];
    const size_t n = (size_t)m.Nx * m.Ny * m.Nz;
    double *tmp = nullptr;
    ck(cudaMallocAsync((void **)&tmp, n * 8, s), "cudaMallocAsync");
    k_unpad<<<1024, 256, 0, s>>>(src, tmp, m.Nx, m.Ny, m.Nz, m.Nzp);
    ck(cudaMemcpyAsync(out, tmp, n * 8, cudaMemcpyDeviceToHost, s), "D2H");
    ck(cudaFreeAsync(tmp, s), "cudaFreeAsync");
}

double *const *Fp32Sim::ntf_arrays() const { return impl_->a.ntf; }

// ---------------------------------------------------------------------------
// Batch of FP32 simulations advanced by the persistent kernel.

// A member's Args in the batch: its own, with the batch's slab depth.  The
// follow-up work (DFT, oblique TF/SF corrections) is k_batch_post's.
static Args batch_args(const Args &a0, int chunk) {
    Args a = a0;
    if (chunk > 0) a.chunk = chunk;
    a.band = 0;  // the batched pass makes the CPML corrections itself
    return a;
}

struct Fp32Batch::Impl {
    int device = 0, sms = 148, jm = -1;
    cudaStream_t stream = nullptr;
    Fp32Sim *slot[kMaxBatch] = {};
    int tsteps[kMaxBatch] = {};
    int host_t[kMaxBatch] = {};     // steps done, mirrored on the host
    BatchItem *items = nullptr;
    int item_cap = 0, n_items = 0;
    int *d_n = nullptr, *d_next = nullptr, *d_t = nullptr, *d_end = nullptr;
    Maps *d_maps = nullptr;
    long long tick = 0;             // global step counter: parity of every slot's pass
    bool dirty = true;
    int chunk = 0;                  // planes per item (0: per-simulation default)
    int ctas_per_sm = 3;            // (at most 2 for the wide path and tabulated Lee-Kalluri: launch_tick)
    int slabk = -1;                 // batch class of the members (Fp32Sim::batch_class); -1: empty
    // class 1: interior tiles 8 x 64 on the wide path (the default: on 24
    // sweep trails 4.86 ms a tick against 5.15 at 8 x 32) or 8 x 32 on the
    // fast path
    int tile_cols = 64;
    int graph_cols = 0;
    Maps *d_mapsw = nullptr;        // the members' maps with the wide path's boxes
    cudaGraphExec_t graph = nullptr;
    int graph_ctas = 0;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    std::vector<std::pair<int, double>> tune_log;  // (chunk * 16 + ctas, ms per tick)

    ~Impl() {
        if (stream) cudaStreamSynchronize(stream);
        if (graph) cudaGraphExecDestroy(graph);
        cudaFree(items); cudaFree(d_n); cudaFree(d_next); cudaFree(d_t); cudaFree(d_end); cudaFree(d_maps);
        cudaFree(d_mapsw);
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
        if (stream) cudaStreamDestroy(stream);
    }
};

int Fp32Batch::capacity() { return kMaxBatch; }

// The kMaxBatch slots of c_jobs belong to a device's copy of this module, so
// every batch on a device draws its members' slots from one pool: two
// batches running at the same time (a server with several batch keys) must
// not write the same slot.  A batch's own per-slot arrays (step, end step,
// maps) are indexed by the same slot numbers and hold zeros elsewhere, so its
// kernels skip the slots of other batches.
namespace {
std::mutex g_slot_mu;
std::map<int, std::vector<char>> g_slot_used;  // device -> slot in use
int take_slot(int device) {
    std::lock_guard<std::mutex> lk(g_slot_mu);
    std::vector<char> &u = g_slot_used[device];
    if (u.empty()) u.assign(kMaxBatch, 0);
    for (int q = 0; q < kMaxBatch; q++)
        if (!u[q]) {
            u[q] = 1;
            return q;
        }
    return -1;
}
void release_slot(int device, int q) {
    std::lock_guard<std::mutex> lk(g_slot_mu);
    std::vector<char> &u = g_slot_used[device];
    if (q >= 0 && q < (int)u.size()) u[q] = 0;
}
}  // namespace

int Fp32Batch::free_slots(int device) {
    std::lock_guard<std::mutex> lk(g_slot_mu);
    auto it = g_slot_used.find(device);
    if (it == g_slot_used.end()) return kMaxBatch;
    int n = 0;
    for (char c : it->second) n += c ? 0 : 1;
    return n;
}

Fp32Batch::Fp32Batch(int device) : impl_(new Impl()) {
    Impl &b = *impl_;
    b.device = device;
    ck(cudaSetDevice(device), "cudaSetDevice");
    cudaDeviceGetAttribute(&b.sms, cudaDevAttrMultiProcessorCount, device);
    ck(cudaStreamCreateWithFlags(&b.stream, cudaStreamNonBlocking), "cudaStreamCreate");
    ck(cudaMalloc(&b.d_n, 4), "cudaMalloc");
    ck(cudaMalloc(&b.d_next, 4), "cudaMalloc");
    ck(cudaMalloc(&b.d_t, 4 * kMaxBatch), "cudaMalloc");
    ck(cudaMalloc(&b.d_end, 4 * kMaxBatch), "cudaMalloc");
    ck(cudaMalloc(&b.d_maps, sizeof(Maps) * kMaxBatch), "cudaMalloc");
    ck(cudaMalloc(&b.d_mapsw, sizeof(Maps) * kMaxBatch), "cudaMalloc");
    ck(cudaMemsetAsync(b.d_n, 0, 4, b.stream), "memset");
    ck(cudaMemsetAsync(b.d_next, 0, 4, b.stream), "memset");
    ck(cudaMemsetAsync(b.d_t, 0, 4 * kMaxBatch, b.stream), "memset");
    ck(cudaMemsetAsync(b.d_end, 0, 4 * kMaxBatch, b.stream), "memset");
    ck(cudaEventCreate(&b.e0), "event");
    ck(cudaEventCreate(&b.e1), "event");
    {
        auto attr = [](const void *f, int bytes) {
            ck(cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes), "attr");
        };
        attr((const void *)k_fp32_batch<0, 0, 0>, SMEM_B); attr((const void *)k_fp32_batch<1, 0, 0>, SMEM_B);
        attr((const void *)k_fp32_batch<0, 1, 0>, SMEM_B); attr((const void *)k_fp32_batch<1, 1, 0>, SMEM_B);
        attr((const void *)k_fp32_batch<0, 2, 0>, SMEM_B); attr((const void *)k_fp32_batch<1, 2, 0>, SMEM_B);
        attr((const void *)k_fp32_batch<0, 0, 1>, SMEM_BS); attr((const void *)k_fp32_batch<1, 0, 1>, SMEM_BS);
        attr((const void *)k_fp32_batch<0, 1, 1>, SMEM_BS); attr((const void *)k_fp32_batch<1, 1, 1>, SMEM_BS);
        auto attrw = [&](const void *f) {
            attr(f, SMEM_BATCHW);
            ck(cudaFuncSetAttribute(f, cudaFuncAttributePreferredSharedMemoryCarveout, 100), "attr");
        };
        attrw((const void *)k_fp32_batch<0, 0, 2>); attrw((const void *)k_fp32_batch<1, 0, 2>);
        attrw((const void *)k_fp32_batch<0, 1, 2>); attrw((const void *)k_fp32_batch<1, 1, 2>);
    }
    ck(cudaStreamSynchronize(b.stream), "batch set-up");
}

Fp32Batch::~Fp32Batch() {
    for (int q = 0; q < kMaxBatch; q++)
        if (impl_->slot[q]) release_slot(impl_->device, q);
    delete impl_;
}

void *Fp32Batch::stream() const { return impl_->stream; }

int Fp32Batch::add(Fp32Sim *sim, int t0) {
    Impl &b = *impl_;
    Fp32Sim::Impl &m = *sim->impl_;
    if (t0 != 0) throw Error(MFDTD_ESTATE, "batch: a simulation joins at step 0");
    if (b.jm >= 0 && m.jm != b.jm)
        throw Error(MFDTD_EINVAL, "batch: every simulation of a batch uses the same current update "
                                  "(Young DI, uniform Lee-Kalluri, or tabulated Lee-Kalluri)");
    const int cls = m.slab_eligible ? 1 : 0;
    if (b.slabk >= 0 && cls != b.slabk)
        throw Error(MFDTD_EINVAL, "batch: every simulation of a batch is of the same batch class (the fast "
                                  "path with the CPML slab march, or the general path)");
    const int s = take_slot(b.device);
    if (s < 0)
        throw Error(MFDTD_ENOMEM, "batch: all " + std::to_string(kMaxBatch) +
                                      " member slots of this device are in use (shared by every batch on it)");
    try {
        ck(cudaStreamSynchronize(b.stream), "batch");
    } catch (...) {
        release_slot(b.device, s);
        throw;
    }
    // The state is all zeros in both sets, so the simulation can take the
    // parity of the current tick.
    sim->m_cur_ = (int)(b.tick & 1);
    if (m.a.nntf > 0 && !m.ntf_ring) {  // the running-DFT ring (k_batch_post)
        try {
            m.ntf_ring = m.alloc<float>((size_t)kNtfRing * 6 * m.nface, b.stream);
        } catch (...) {
            release_slot(b.device, s);
            throw;
        }
        sim->bytes_ = m.bytes;
    }
    m.ring_fill = 0;
    // (in the simulation's own Args, so that every later copy into the
    // constant bank -- apply_chunk -- carries it)
    m.a.ntf_ring = m.ntf_ring;
    const Args ba = batch_args(m.a, 0);
    ck(cudaMemcpyToSymbolAsync(c_jobs, &ba, sizeof(Args), sizeof(Args) * s, cudaMemcpyHostToDevice, b.stream),
       "cudaMemcpyToSymbol");
    ck(cudaMemcpyAsync(b.d_maps + s, &m.maps, sizeof(Maps), cudaMemcpyHostToDevice, b.stream), "H2D");
    ck(cudaMemcpyAsync(b.d_mapsw + s, &m.mapsw, sizeof(Maps), cudaMemcpyHostToDevice, b.stream), "H2D");
    int zero = 0, end = m.tsteps;
    ck(cudaMemcpyAsync(b.d_t + s, &zero, 4, cudaMemcpyHostToDevice, b.stream), "H2D");
    ck(cudaMemcpyAsync(b.d_end + s, &end, 4, cudaMemcpyHostToDevice, b.stream), "H2D");
    ck(cudaStreamSynchronize(b.stream), "batch add");
    b.slot[s] = sim;
    b.tsteps[s] = m.tsteps;
    b.host_t[s] = 0;
    b.jm = m.jm;
    if (b.slabk != cls) {
        b.slabk = cls;
        if (b.graph) { cudaGraphExecDestroy(b.graph); b.graph = nullptr; }
    }
    b.dirty = true;
    return s;
}

void Fp32Batch::remove(Fp32Sim *sim) {
    Impl &b = *impl_;
    for (int q = 0; q < kMaxBatch; q++)
        if (b.slot[q] == sim) {
            ck(cudaStreamSynchronize(b.stream), "batch");
            int zero = 0;
            ck(cudaMemcpy(b.d_end + q, &zero, 4, cudaMemcpyHostToDevice), "H2D");
            // DFT steps still in the ring (the member leaves before its last
            // step, off a ring boundary) go to the sums now
            Fp32Sim::Impl &m = *sim->impl_;
            const int done = b.host_t[q], pend = done % kNtfRing;
            if (m.ntf_ring && pend && done < b.tsteps[q]) {
                m.ring_t0 = done - pend;
                m.ring_fill = pend;
                sim->drain_ntf(b.stream);
                ck(cudaStreamSynchronize(b.stream), "batch");
            }
            b.slot[q] = nullptr;
            release_slot(b.device, q);
            b.dirty = true;
        }
    bool any = false;
    for (int q = 0; q < kMaxBatch; q++) any |= b.slot[q] != nullptr;
    if (!any) {
        b.jm = -1;
        b.slabk = -1;
    }
}

int Fp32Batch::steps_done(const Fp32Sim *sim) const {
    for (int q = 0; q < kMaxBatch; q++)
        if (impl_->slot[q] == sim) return impl_->host_t[q];
    return -1;
}

// Work items of every simulation still short of its step count, each tile
// split into x-chunks (the slab depth).  In a batch of class 1 every member is
// marched like a single simulation: its interior tiles on the fast path over
// the interior planes and by the slab march over the x-slab planes, its other
// tiles by the slab march over every plane.  In a batch of class 0 every item
// takes the general path (boundary tiles first).  Order: slab marches of whole
// tile columns and general boundary tiles (the slow items), then fast and
// general interior items, then the short x-slab items.
static void build_items(Fp32Batch::Impl &b) {
    std::vector<BatchItem> slow, mid, tail;
    for (int q = 0; q < kMaxBatch; q++) {
        Fp32Sim *sim = b.slot[q];
        if (!sim || b.host_t[q] >= b.tsteps[q]) continue;
        Fp32Sim::Impl &m = *sim->impl();
        const int chunk = b.chunk > 0 ? b.chunk : m.a.chunk;
        const int Nx = m.Nx;
        bool first = true;
        auto add = [&](std::vector<BatchItem> &v, int tile, int ib, int ie, int mode) {
            for (int c0 = ib; c0 < ie; c0 += chunk) {
                BatchItem w{};
                w.job = q;
                w.tile = tile;
                w.ib = (unsigned short)c0;
                w.ie = (unsigned short)std::min(ie, c0 + chunk);
                w.mode = (unsigned char)mode;
                w.yz = (unsigned char)(mode == MARCH_SLAB ? slab_yz(m, tile) : 3);
                w.first = first ? 1 : 0;
                first = false;
                v.push_back(w);
            }
        };
        if (b.slabk == 1 && b.tile_cols == 64) {
            for (int tl : m.edgew) add(slow, tl, 0, Nx, MARCH_SLAB);
            for (int tl : m.pairs32) add(mid, tl, 0, Nx, MARCH_WIDE);
        } else if (b.slabk == 1) {
            const int w = m.wband;
            for (int tl : m.edge32) add(slow, tl, 0, Nx, MARCH_SLAB);
            for (int tl : m.inner32) add(mid, tl, w, Nx - w, MARCH_FAST);
            for (int tl : m.inner32) {
                add(tail, tl, 0, w, MARCH_SLAB);
                add(tail, tl, Nx - w, Nx, MARCH_SLAB);
            }
        } else {
            for (size_t ti = 0; ti < m.tile_order.size(); ti++)
                add((int)ti < m.n_boundary ? slow : mid, m.tile_order[ti], 0, Nx, MARCH_GENERAL);
        }
    }
    std::vector<BatchItem> all;
    all.reserve(slow.size() + mid.size() + tail.size());
    all.insert(all.end(), slow.begin(), slow.end());
    all.insert(all.end(), mid.begin(), mid.end());
    all.insert(all.end(), tail.begin(), tail.end());
    if ((int)all.size() > b.item_cap) {
        cudaFree(b.items);
        b.item_cap = (int)all.size() * 2 + 1024;
        ck(cudaMalloc(&b.items, sizeof(BatchItem) * b.item_cap), "cudaMalloc");
        if (b.graph) { cudaGraphExecDestroy(b.graph); b.graph = nullptr; }
    }
    b.n_items = (int)all.size();
    if (b.n_items)
        ck(cudaMemcpyAsync(b.items, all.data(), sizeof(BatchItem) * b.n_items, cudaMemcpyHostToDevice,
                           b.stream), "H2D");
    ck(cudaMemcpyAsync(b.d_n, &b.n_items, 4, cudaMemcpyHostToDevice, b.stream), "H2D");
    b.dirty = false;
}

// The simulations' chunk length is written into their constant slots (Args).
static void apply_chunk(Fp32Batch::Impl &b) {
    for (int q = 0; q < kMaxBatch; q++) {
        Fp32Sim *sim = b.slot[q];
        if (!sim) continue;
        const Args a = batch_args(sim->impl()->a, b.chunk);
        ck(cudaMemcpyToSymbolAsync(c_jobs, &a, sizeof(Args), sizeof(Args) * q, cudaMemcpyHostToDevice,
                                   b.stream), "cudaMemcpyToSymbol");
    }
}

static int batch_kind(const Fp32Batch::Impl &b) { return b.slabk == 1 ? (b.tile_cols == 64 ? 2 : 1) : 0; }

static void launch_tick(Fp32Batch::Impl &b, int par) {
    const int kind = batch_kind(b);
    // the kernels of the wide path and of tabulated Lee-Kalluri fit two CTAs per SM
    const int cap = (kind == 2 || b.jm == 2) ? 2 : 3;
    const dim3 grid(b.sms * std::min(b.ctas_per_sm, cap));
    const int smem = kind == 2 ? SMEM_BATCHW : kind == 1 ? SMEM_BS : SMEM_B;
    auto go = [&](auto kern) {
        kern<<<grid, NTHREADS, smem, b.stream>>>(b.items, b.d_n, b.d_next, b.d_maps, b.d_mapsw, b.d_t, b.d_end);
    };
    if (par == 0) {
        if (b.jm == 0) kind == 2 ? go(k_fp32_batch<0, 0, 2>) : kind == 1 ? go(k_fp32_batch<0, 0, 1>) : go(k_fp32_batch<0, 0, 0>);
        else if (b.jm == 1) kind == 2 ? go(k_fp32_batch<0, 1, 2>) : kind == 1 ? go(k_fp32_batch<0, 1, 1>) : go(k_fp32_batch<0, 1, 0>);
        else go(k_fp32_batch<0, 2, 0>);
    } else {
        if (b.jm == 0) kind == 2 ? go(k_fp32_batch<1, 0, 2>) : kind == 1 ? go(k_fp32_batch<1, 0, 1>) : go(k_fp32_batch<1, 0, 0>);
        else if (b.jm == 1) kind == 2 ? go(k_fp32_batch<1, 1, 2>) : kind == 1 ? go(k_fp32_batch<1, 1, 1>) : go(k_fp32_batch<1, 1, 0>);
        else go(k_fp32_batch<1, 2, 0>);
    }
    const dim3 pgrid(b.sms, kMaxBatch);
    if (par == 0) k_batch_post<0><<<pgrid, 256, 0, b.stream>>>(b.d_t, b.d_end);
    else k_batch_post<1><<<pgrid, 256, 0, b.stream>>>(b.d_t, b.d_end);
    k_batch_flush<<<pgrid, 256, 0, b.stream>>>(b.d_t, b.d_end);
    k_batch_advance<<<1, kMaxBatch, 0, b.stream>>>(b.d_t, b.d_end, kMaxBatch, b.d_next);
}

// Two ticks (one of each parity) captured once and replayed.
static void ensure_graph(Fp32Batch::Impl &b) {
    if (b.graph && b.graph_ctas == b.ctas_per_sm && b.graph_cols == b.tile_cols) return;
    if (b.graph) { cudaGraphExecDestroy(b.graph); b.graph = nullptr; }
    cudaGraph_t g;
    ck(cudaStreamBeginCapture(b.stream, cudaStreamCaptureModeThreadLocal), "capture");
    launch_tick(b, 0);
    launch_tick(b, 1);
    ck(cudaStreamEndCapture(b.stream, &g), "capture");
    ck(cudaGraphInstantiate(&b.graph, g, 0), "cudaGraphInstantiate");
    cudaGraphDestroy(g);
    b.graph_ctas = b.ctas_per_sm;
    b.graph_cols = b.tile_cols;
}

int Fp32Batch::run(int nticks) {
    Impl &b = *impl_;
    if (b.jm < 0 || nticks <= 0) return 0;
    if (b.dirty) build_items(b);
    int launches = 0;
    int done = 0;
    // A tick of odd parity first, so that the graph (even, odd) starts even.
    constexpr int kPerTick = 3;  // batched pass, follow-up work, advance
    if (b.tick & 1) { launch_tick(b, 1); b.tick++; done++; launches += kPerTick; }
    if (nticks - done >= 2) ensure_graph(b);
    while (nticks - done >= 2) {
        ck(cudaGraphLaunch(b.graph, b.stream), "cudaGraphLaunch");
        b.tick += 2; done += 2; launches += 2 * kPerTick;
    }
    if (done < nticks) { launch_tick(b, (int)(b.tick & 1)); b.tick++; done++; launches += kPerTick; }
    ck(cudaGetLastError(), "batch launch");
    for (int q = 0; q < kMaxBatch; q++)
        if (b.slot[q]) {
            const int before = b.host_t[q];
            b.host_t[q] = std::min(b.tsteps[q], before + nticks);
            // every pass flips the simulation's current set
            if ((b.host_t[q] - before) & 1) b.slot[q]->m_cur_ ^= 1;
            if (b.host_t[q] >= b.tsteps[q] && before < b.tsteps[q]) b.dirty = true;
        }
    return launches;
}

void Fp32Batch::sync() {
    ck(cudaStreamSynchronize(impl_->stream), "batch sync");
    for (int q = 0; q < kMaxBatch; q++)
        if (impl_->slot[q]) impl_->slot[q]->check(impl_->stream);
}

// Online autotuning: each candidate (slab depth, CTAs per SM) advances the
// live batch by two ticks, timed with events; the fastest candidate is kept.
// The work is not wasted -- the simulations advance -- so the tuner costs
// only the ticks spent on slower settings.
int Fp32Batch::tune(const int *chunks, int nchunks, const int *ctas, int nctas) {
    Impl &b = *impl_;
    if (b.jm < 0) return 0;
    double best = 1e300;
    int best_chunk = b.chunk, best_ctas = b.ctas_per_sm, best_cols = b.tile_cols, ticks = 0;
    b.tune_log.clear();
    // tile shapes: 8 x 32 everywhere, or (slab class) interior tiles paired
    // into 8 x 64 on the wide path, at most two CTAs per SM
    const int shapes[2] = {32, 64};
    const int nshapes = b.slabk == 1 ? 2 : 1;
    for (int si = 0; si < nshapes; si++)
        for (int ci = 0; ci < nchunks; ci++)
            for (int ki = 0; ki < nctas; ki++) {
                int left = 1 << 30;
                for (int q = 0; q < kMaxBatch; q++)
                    if (b.slot[q]) left = std::min(left, b.tsteps[q] - b.host_t[q]);
                if (left < 4) break;
                const int cap = (b.jm == 2 || shapes[si] == 64) ? 2 : 3;
                if (ctas[ki] > cap && nctas > 1) continue;  // that occupancy does not exist for the shape
                b.tile_cols = shapes[si];
                b.chunk = chunks[ci];
                b.ctas_per_sm = std::max(1, std::min(ctas[ki], cap));
                apply_chunk(b);
                b.dirty = true;
                run(2);  // settle (graph capture, item rebuild)
                ck(cudaEventRecord(b.e0, b.stream), "event");
                run(2);
                ck(cudaEventRecord(b.e1, b.stream), "event");
                ck(cudaEventSynchronize(b.e1), "event");
                float ms = 0;
                cudaEventElapsedTime(&ms, b.e0, b.e1);
                b.tune_log.push_back({(b.tile_cols * 1024 + chunks[ci]) * 16 + b.ctas_per_sm, ms / 2});
                ticks += 4;
                if (ms < best) {
                    best = ms;
                    best_chunk = b.chunk;
                    best_ctas = b.ctas_per_sm;
                    best_cols = b.tile_cols;
                }
            }
    b.chunk = best_chunk;
    b.ctas_per_sm = best_ctas;
    b.tile_cols = best_cols;
    apply_chunk(b);
    b.dirty = true;
    return ticks;
}

int Fp32Batch::tuned_tile_cols() const { return impl_->tile_cols; }
int Fp32Batch::tuned_chunk() const { return impl_->chunk; }
int Fp32Batch::impl_device() const { return impl_->device; }
int Fp32Batch::tuned_ctas() const { return impl_->ctas_per_sm; }
long long Fp32Batch::tick() const { return impl_->tick; }

Fp32Sim::~Fp32Sim() { delete impl_; }

}  // namespace mfdtd
