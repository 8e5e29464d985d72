// farfield.cu -- near-to-far-field projection of the Huygens-surface sums.
//
// Generalises analysis/meteorNTF.m:236-332 (backscatter only, observer along
// -x) to any set of directions r_hat(theta, phi):
//     L(r_hat) = sum over the 12 M arrays, N(r_hat) = sum over the 12 J arrays of
//     w * dA * X(a,b) * exp(-j k r_hat . r'(a,b)),
// where X = cos-sum + 1i * sin-sum is the phasor of one DFT accumulator
// (analysis/meteorNTF.m:202-230), w the trapezoid edge weight and r' the Yee
// position of the sample (the half-cell offsets of meteorNTF.m:236-246).
//
// The phase factor of a sample on a face with in-plane axes (a, b) separates,
// exp(-jk r_n n0) * exp(-jk r_a pos_a) * exp(-jk r_b pos_b), so per face:
//   stage 1 (complex GEMM): T[u][a] = sum_b P[u][b] X[a][b],
//            P[u][b] = w_b exp(-jk s_u pos_b), s_u the distinct values of r_b
//            over the direction set (a theta/phi grid has few of them);
//   stage 2 (reduction):    L[d] += exp(-jk r_n n0) dA sum_a w_a exp(-jk r_a pos_a) T[u(d)][a].
// Method 0 runs both stages in FP64 on the CUDA cores.  Method 1 runs stage 1
// -- the dense contraction; on the faces whose b axis is y there is one u per
// direction, so it is a full GEMM -- on the tensor cores (tcgen05, TF32 with
// FP32 accumulation).  Each operand is split into a TF32 head and a TF32
// tail, x = hi + lo, and the three significant products hi*hi + hi*lo + lo*hi
// are accumulated in one GEMM by concatenating the splits along K, which
// keeps about 21 bits per product.  The complex product is one real GEMM:
// rows [Pr | Pi] of the phase against rows [Xr | -Xi] (real part) and
// [Xi | Xr] (imaginary part) of the sums.  Stage 2 stays FP64.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "common.hpp"
#include "farfield.hpp"
#include "tc_gemm.cuh"

namespace mfdtd {
namespace {

constexpr double kPI = 3.141592653589793;
// analysis/loadconstants.m:3-10 (the RCS post-processing constants)
const double kU0a = 4 * kPI * 1e-7, kE0a = 8.845e-12;

void ck(cudaError_t e, const char *what) {
    if (e != cudaSuccess) throw Error(MFDTD_ECUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

// P[u][b] = w_b * exp(-j k s_u pos_b)
__global__ void k_ff_phase(double2 *P, const double *s, int U, int B, double k, double b_off,
                           double hb, int halve_ends) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x, u = blockIdx.y;
    if (b >= B || u >= U) return;
    const double pos = (b + b_off) * hb;
    double sn, cs;
    sincos(-k * s[u] * pos, &sn, &cs);
    const double w = (halve_ends && (b == 0 || b == B - 1)) ? 0.5 : 1.0;
    P[(size_t)u * B + b] = make_double2(w * cs, w * sn);
}

// T[u][a] = sum_b P[u][b] * X(a, b); X(a,b) = src[((a0+a)*Bs + b0+b)*n2 + 2m + {1: re, 0: im}]
constexpr int FT = 16;
__global__ void __launch_bounds__(256) k_ff_gemm(double2 *T, const double2 *P, const double *src,
                                                 int U, int A, int B, int a0, int b0, int Bs, int n2,
                                                 int m) {
    __shared__ double2 Ps[FT][FT + 1];
    __shared__ double2 Xs[FT][FT + 1];
    const int tx = threadIdx.x, ty = threadIdx.y;  // tx: a within tile, ty: u within tile
    const int a = blockIdx.x * FT + tx, u = blockIdx.y * FT + ty;
    double re = 0, im = 0;
    for (int bb = 0; bb < B; bb += FT) {
        // P tile: rows u, cols b ; X tile: rows a, cols b
        {
            const int uu = blockIdx.y * FT + ty, b = bb + tx;
            Ps[ty][tx] = (uu < U && b < B) ? P[(size_t)uu * B + b] : make_double2(0, 0);
            const int aa = blockIdx.x * FT + ty;
            if (aa < A && b < B) {
                const size_t o = ((size_t)(a0 + aa) * Bs + (b0 + b)) * n2 + 2 * m;
                Xs[ty][tx] = make_double2(src[o + 1], src[o]);
            } else {
                Xs[ty][tx] = make_double2(0, 0);
            }
        }
        __syncthreads();
#pragma unroll
        for (int q = 0; q < FT; q++) {
            const double2 p = Ps[ty][q], x = Xs[tx][q];
            re += p.x * x.x - p.y * x.y;
            im += p.x * x.y + p.y * x.x;
        }
        __syncthreads();
    }
    if (a < A && u < U) T[(size_t)u * A + a] = make_double2(re, im);
}

// out[d] += scale(d) * sum_a w_a exp(-jk r_a(d) pos_a) T[u(d)][a]
__global__ void __launch_bounds__(256) k_ff_reduce(double2 *out, const double2 *T, const int *umap,
                                                   const double *ra, const double *rn, int D, int A,
                                                   double k, double a_off, double ha, int halve_ends,
                                                   double n0, double area) {
    const int d = blockIdx.x;
    if (d >= D) return;
    const double2 *row = T + (size_t)umap[d] * A;
    const double kr = -k * ra[d];
    double re = 0, im = 0;
    for (int a = threadIdx.x; a < A; a += blockDim.x) {
        double sn, cs;
        sincos(kr * ((a + a_off) * ha), &sn, &cs);
        const double w = (halve_ends && (a == 0 || a == A - 1)) ? 0.5 : 1.0;
        const double2 t = row[a];
        re += w * (cs * t.x - sn * t.y);
        im += w * (cs * t.y + sn * t.x);
    }
    for (int off = 16; off > 0; off >>= 1) {
        re += __shfl_down_sync(0xffffffffu, re, off);
        im += __shfl_down_sync(0xffffffffu, im, off);
    }
    __shared__ double sre[8], sim[8];
    if ((threadIdx.x & 31) == 0) { sre[threadIdx.x >> 5] = re; sim[threadIdx.x >> 5] = im; }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < (int)(blockDim.x >> 5); w++) { re += sre[w]; im += sim[w]; }
        double sn, cs;
        sincos(-k * rn[d] * n0, &sn, &cs);
        const double xr = area * (cs * re - sn * im), xi = area * (cs * im + sn * re);
        out[d].x += xr;
        out[d].y += xi;
    }
}

// ---- tensor-core stage 1 -----------------------------------------------------
__device__ __forceinline__ float tf32_round(float x) {
    return __uint_as_float((__float_as_uint(x) + 0x1000u) & ~0x1FFFu);
}
// TF32 head and tail of an FP64 value: hi + lo carries about 21 bits.
__device__ __forceinline__ void tf32_split(double v, float &hi, float &lo) {
    hi = tf32_round((float)v);
    lo = tf32_round((float)(v - (double)hi));
}

// sin and cos of an FP64 phase: the argument is reduced to [-pi, pi] in FP64
// and evaluated in FP32 (about 23 bits, more than the 21 the TF32 split keeps;
// FP64 transcendentals are slow on this part).
__device__ __forceinline__ void sincos_reduced(double x, float *sn, float *cs) {
    const double two_pi = 6.283185307179586;
    const double r = x - two_pi * rint(x * (1.0 / two_pi));
    sincosf((float)r, sn, cs);
}

// Phase operand: row u, K = [Phi_r Phi_i | Phi_r Phi_i | Plo_r Plo_i] (B each),
// zero-padded to Kpad and to Upad rows.  One thread per (u, b).
__global__ void k_tc_pack_phase(float *A, const double *s, int U, int B, int Kpad, double k,
                                double b_off, double hb, int halve_ends) {
    const int u = blockIdx.y;
    float *row = A + (size_t)u * Kpad;
    for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < B; b += gridDim.x * blockDim.x) {
        float rh = 0.f, rl = 0.f, ih = 0.f, il = 0.f;
        if (u < U) {
            const double pos = (b + b_off) * hb;
            float sn, cs;
            sincos_reduced(-k * s[u] * pos, &sn, &cs);
            const double w = (halve_ends && (b == 0 || b == B - 1)) ? 0.5 : 1.0;
            tf32_split(w * (double)cs, rh, rl);
            tf32_split(w * (double)sn, ih, il);
        }
        row[b] = rh; row[B + b] = ih;              // meets the sums head
        row[2 * B + b] = rh; row[3 * B + b] = ih;  // meets the sums tail
        row[4 * B + b] = rl; row[5 * B + b] = il;  // phase tail, meets the sums head
    }
    for (int q = 6 * B + blockIdx.x * blockDim.x + threadIdx.x; q < Kpad; q += gridDim.x * blockDim.x)
        row[q] = 0.f;
}

// Sums operand: row r = c * 2A + 2a + {0 re, 1 im} for the components c of one
// face kind, K = [X_hi | X_lo | X_hi] with the real row [Xr, -Xi] and the
// imaginary row [Xi, Xr]; X(a,b) = cos-sum + i sin-sum of the DFT arrays.
struct PackSrc {
    const double *src[2];
};
__global__ void k_tc_pack_sums(float *Bm, PackSrc ps, int ncomp, int A, int B, int a0, int b0, int Bs,
                               int n2, int m, int Kpad) {
    const int r = blockIdx.y;
    const int c = r / (2 * A), a = (r % (2 * A)) / 2, im = r & 1;
    float *row = Bm + (size_t)r * Kpad;
    for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < B; b += gridDim.x * blockDim.x) {
        float h0 = 0.f, l0 = 0.f, h1 = 0.f, l1 = 0.f;
        if (c < ncomp) {
            const size_t o = ((size_t)(a0 + a) * Bs + (b0 + b)) * n2 + 2 * m;
            const double xr = ps.src[c][o + 1], xi = ps.src[c][o];
            tf32_split(im ? xi : xr, h0, l0);    // first half of each segment
            tf32_split(im ? xr : -xi, h1, l1);   // second half
        }
        row[b] = h0; row[B + b] = h1;              // meets the phase head
        row[2 * B + b] = l0; row[3 * B + b] = l1;  // sums tail, meets the phase head
        row[4 * B + b] = h0; row[5 * B + b] = h1;  // meets the phase tail
    }
    for (int q = 6 * B + blockIdx.x * blockDim.x + threadIdx.x; q < Kpad; q += gridDim.x * blockDim.x)
        row[q] = 0.f;
}

// Stage 2 reading stage 1 from the FP32 GEMM tile: T[u][a] = (C[u][col0 + 2a],
// C[u][col0 + 2a + 1]).  One warp per direction (faces are a few hundred cells
// wide).  Lane l takes a = l, l + 32, ...: its first phase and the phase step
// of 32 cells are reduced in FP64 once, and the phasor then advances by FP32
// complex rotation (a dozen steps on a face of a few hundred cells, about 1e-6
// rad of drift, the order of the stage-1 split's own error).  The terms and
// the lanes' partial sums are FP32 like the stage-1 result they weight; the
// face factor is applied in FP64.  (FP64
// arithmetic per term ran at this part's reduced FP64 rate: 0.24 ms a
// launch on a 384^3 grid at 16,380 directions.)
__global__ void __launch_bounds__(256) k_ff_reduce_tc(double2 *out, const float *C, int ldc, int col0,
                                                      const int *umap, const double *ra, const double *rn,
                                                      int D, int A, double k, double a_off, double ha,
                                                      int halve_ends, double n0, double area) {
    const int d = blockIdx.x * 8 + (threadIdx.x >> 5), lane = threadIdx.x & 31;
    if (d >= D) return;
    const float2 *row = (const float2 *)(C + (size_t)umap[d] * ldc + col0);
    const double kr = -k * ra[d];
    float sn, cs, sd, cd;
    sincos_reduced(kr * ((lane + a_off) * ha), &sn, &cs);
    sincos_reduced(kr * (32.0 * ha), &sd, &cd);
    float fre = 0.f, fim = 0.f;
    for (int a = lane; a < A; a += 32) {
        const float w = (halve_ends && (a == 0 || a == A - 1)) ? 0.5f : 1.0f;
        const float2 t = row[a];
        fre += w * (cs * t.x - sn * t.y);
        fim += w * (cs * t.y + sn * t.x);
        const float cn = cs * cd - sn * sd;
        sn = sn * cd + cs * sd;
        cs = cn;
    }
    for (int off = 16; off > 0; off >>= 1) {
        fre += __shfl_down_sync(0xffffffffu, fre, off);
        fim += __shfl_down_sync(0xffffffffu, fim, off);
    }
    const double re = fre, im = fim;
    if (lane == 0) {
        float sn, cs;
        sincos_reduced(-k * rn[d] * n0, &sn, &cs);
        out[d].x += area * ((double)cs * re - (double)sn * im);
        out[d].y += area * ((double)cs * im + (double)sn * re);
    }
}

// sigma of every direction from the six accumulated vector potentials (L, N
// along x, y, z, each `stride` directions apart), analysis/meteorNTF.m:311-332
// generalised to (theta, phi); c = k^2 / (8 pi eta0) / P_inc.
__global__ void k_ff_sigma(const double2 *acc, size_t stride, const double *th, const double *ph, int n,
                           double c, double eta0, double *sig) {
    const int d = blockIdx.x * blockDim.x + threadIdx.x;
    if (d >= n) return;
    auto g = [&](int q) { return acc[(size_t)q * stride + d]; };
    const double2 Lx = g(0), Ly = g(1), Lz = g(2), Nx = g(3), Ny = g(4), Nz = g(5);
    double stt, ct, sp, cp;
    sincos(th[d], &stt, &ct);
    sincos(ph[d], &sp, &cp);
    const double Lthr = Lx.x * ct * cp + Ly.x * ct * sp - Lz.x * stt, Lthi = Lx.y * ct * cp + Ly.y * ct * sp - Lz.y * stt;
    const double Lphr = -Lx.x * sp + Ly.x * cp, Lphi = -Lx.y * sp + Ly.y * cp;
    const double Nthr = Nx.x * ct * cp + Ny.x * ct * sp - Nz.x * stt, Nthi = Nx.y * ct * cp + Ny.y * ct * sp - Nz.y * stt;
    const double Nphr = -Nx.x * sp + Ny.x * cp, Nphi = -Nx.y * sp + Ny.y * cp;
    const double ar = Lphr + eta0 * Nthr, ai = Lphi + eta0 * Nthi;
    const double br = Lthr - eta0 * Nphr, bi = Lthi - eta0 * Nphi;
    const double sa = c * (ar * ar + ai * ai), sb = c * (br * br + bi * bi);
    sig[3 * d] = sa + sb;
    sig[3 * d + 1] = sa;
    sig[3 * d + 2] = sb;
}

using EncodeFn = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                              const cuuint64_t *, const cuuint32_t *, const cuuint32_t *,
                              CUtensorMapInterleave, CUtensorMapSwizzle, CUtensorMapL2promotion,
                              CUtensorMapFloatOOBfill);
EncodeFn tensor_map_encoder() {
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

// K-major operand [rows][Kpad] fp32, 128 x 32 boxes with 128-byte swizzling.
void tc_operand_map(CUtensorMap *m, float *base, int rows, int Kpad) {
    cuuint64_t dims[2] = {(cuuint64_t)Kpad, (cuuint64_t)rows};
    cuuint64_t strides[1] = {(cuuint64_t)Kpad * 4};
    cuuint32_t box[2] = {(cuuint32_t)tc::BK, 128}, es[2] = {1, 1};
    CUresult r = tensor_map_encoder()(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, base, dims, strides, box, es,
                                      CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                                      CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) throw Error(MFDTD_ECUDA, "cuTensorMapEncodeTiled failed: " + std::to_string((int)r));
}

struct FaceDesc {
    int n_ax, a_ax, b_ax;  // 0 = x, 1 = y, 2 = z
    bool high;             // back / top / right
};
// face order in the NTF arrays: front, back, top, bot, left, right
const FaceDesc kFaces[6] = {{0, 1, 2, false}, {0, 1, 2, true}, {1, 0, 2, true},
                            {1, 0, 2, false}, {2, 0, 1, false}, {2, 0, 1, true}};
// per face: (array offset within the face's 4, vector 0=M/1=J, field axis, kind 0=A/1=B)
struct CompDesc {
    int q, vec, axis, kind;
};
// arrays of one face in file order: front: My, Mz, Jy, Jz ; top: Mx, Mz, Jx, Jz ; left: Mx, My, Jx, Jy
const CompDesc kComps[3][4] = {
    {{0, 0, 1, 0}, {1, 0, 2, 1}, {2, 1, 1, 1}, {3, 1, 2, 0}},   // x faces
    {{0, 0, 0, 0}, {1, 0, 2, 1}, {2, 1, 0, 1}, {3, 1, 2, 0}},   // y faces
    {{0, 0, 0, 0}, {1, 0, 1, 1}, {2, 1, 0, 1}, {3, 1, 1, 0}}};  // z faces

}  // namespace

// Far-field of the 24 device arrays `ntf` (file layout) for the given directions.
void far_field_fp64(const Problem &P, double *const ntf[24], const double *srcdft, int ndir,
                    const double *theta, const double *phi, double *out, void *stream, int method) {
    cudaStream_t st = (cudaStream_t)stream;
    if (method == 1) {
        static bool attr_done = false;
        if (!attr_done) {
            ck(cudaFuncSetAttribute(tc::k_tc_gemm_tf32, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    tc::SMEM_BYTES), "attr");
            attr_done = true;
        }
    }
    const int nf = P.nntf(), ntfb = P.ntfb, n2 = 2 * nf;
    const int dims[3] = {P.Nx, P.Ny, P.Nz};
    const double h[3] = {P.dx, P.dy, P.dz};
    const double vp = std::sqrt(1.0 / (kU0a * kE0a)), eta0 = std::sqrt(kU0a / kE0a);
    std::vector<double> r[3];
    for (int q = 0; q < 3; q++) r[q].resize(ndir);
    for (int d = 0; d < ndir; d++) {
        r[0][d] = std::sin(theta[d]) * std::cos(phi[d]);
        r[1][d] = std::sin(theta[d]) * std::sin(phi[d]);
        r[2][d] = std::cos(theta[d]);
    }
    double *d_r[3];
    std::vector<void *> tmp;
    auto dmalloc = [&](size_t bytes) {
        void *p = nullptr;
        ck(cudaMallocAsync(&p, std::max<size_t>(bytes, 8), st), "cudaMallocAsync");
        tmp.push_back(p);
        return p;
    };
    for (int q = 0; q < 3; q++) {
        d_r[q] = (double *)dmalloc(ndir * 8);
        ck(cudaMemcpyAsync(d_r[q], r[q].data(), ndir * 8, cudaMemcpyHostToDevice, st), "H2D");
    }
    // accumulators [freq][vec][axis][dir]
    double2 *acc = (double2 *)dmalloc((size_t)nf * 6 * ndir * sizeof(double2));
    ck(cudaMemsetAsync(acc, 0, (size_t)nf * 6 * ndir * sizeof(double2), st), "memset");
    // tensor-core GEMM timeout flag (method 1), read once after every launch
    unsigned int *err = (unsigned int *)dmalloc(4);
    ck(cudaMemsetAsync(err, 0, 4, st), "memset");

    // Distinct direction cosines along each axis (u), and the map d -> u.
    // Stage 1 runs over u only: on a regular theta/phi grid far fewer values
    // than directions.  Faces whose in-plane b axis is the same share them.
    std::vector<double> svals[3];
    std::vector<int> umaps[3];
    double *d_sv[3];
    int *d_um[3];
    for (int ax = 0; ax < 3; ax++) {
        std::vector<int> order(ndir);
        for (int d = 0; d < ndir; d++) order[d] = d;
        std::sort(order.begin(), order.end(), [&](int x, int y) { return r[ax][x] < r[ax][y]; });
        umaps[ax].resize(ndir);
        for (int q = 0; q < ndir; q++) {
            const double v = r[ax][order[q]];
            if (svals[ax].empty() || v != svals[ax].back()) svals[ax].push_back(v);
            umaps[ax][order[q]] = (int)svals[ax].size() - 1;
        }
        d_sv[ax] = (double *)dmalloc(svals[ax].size() * 8);
        d_um[ax] = (int *)dmalloc(ndir * 4);
        ck(cudaMemcpyAsync(d_sv[ax], svals[ax].data(), svals[ax].size() * 8, cudaMemcpyHostToDevice, st), "H2D");
        ck(cudaMemcpyAsync(d_um[ax], umaps[ax].data(), ndir * 4, cudaMemcpyHostToDevice, st), "H2D");
    }

    for (int f = 0; f < 6; f++) {
        const FaceDesc &F = kFaces[f];
        const int Na = dims[F.a_ax], Nb = dims[F.b_ax];
        const int U = (int)svals[F.b_ax].size();
        const double *d_s = d_sv[F.b_ax];
        const int *d_umap = d_um[F.b_ax];
        const double n0 = (F.high ? dims[F.n_ax] - ntfb : ntfb) * h[F.n_ax];
        const double area = h[F.a_ax] * h[F.b_ax];
        // trims (analysis/meteorNTF.m:66-196): type A keeps a in [ntfb, Na-ntfb]
        // (ends halved) and b in [ntfb, Nb-ntfb-1] at half-integer positions;
        // type B keeps a in [ntfb, Na-ntfb-1] at half-integer positions and b in
        // [ntfb, Nb-ntfb] (ends halved).
        for (int kind = 0; kind < 2; kind++) {
            const int A = kind == 0 ? Na - 2 * ntfb + 1 : Na - 2 * ntfb;
            const int B = kind == 0 ? Nb - 2 * ntfb : Nb - 2 * ntfb + 1;
            if (A <= 0 || B <= 0) continue;
            const double a_off = kind == 0 ? ntfb : ntfb + 0.5;
            const double b_off = kind == 0 ? ntfb + 0.5 : ntfb;
            if (method == 1) {
                // stage 1 on the tensor cores, both components of this kind at once
                const CompDesc *cs[2];
                int ncomp = 0;
                for (int c = 0; c < 4; c++)
                    if (kComps[F.n_ax][c].kind == kind) cs[ncomp++] = &kComps[F.n_ax][c];
                const int Upad = (U + 127) / 128 * 128, Nrows = ncomp * 2 * A;
                const int Npad = (Nrows + 127) / 128 * 128, Kpad = (6 * B + 31) / 32 * 32;
                float *Am = (float *)dmalloc((size_t)Upad * Kpad * 4);
                float *Bm = (float *)dmalloc((size_t)Npad * Kpad * 4);
                float *Cm = (float *)dmalloc((size_t)Upad * Npad * 4);
                CUtensorMap ma, mb;
                tc_operand_map(&ma, Am, Upad, Kpad);
                tc_operand_map(&mb, Bm, Npad, Kpad);
                PackSrc ps{{ntf[f * 4 + cs[0]->q], ntf[f * 4 + cs[ncomp > 1 ? 1 : 0]->q]}};
                for (int m = 0; m < nf; m++) {
                    const double k = 2 * kPI * P.fntf[m] / vp;
                    k_tc_pack_phase<<<dim3((B + 127) / 128, Upad), 128, 0, st>>>(
                        Am, d_s, U, B, Kpad, k, b_off, h[F.b_ax], kind == 1);
                    k_tc_pack_sums<<<dim3((B + 127) / 128, Npad), 128, 0, st>>>(
                        Bm, ps, ncomp, A, B, ntfb, ntfb, Nb, n2, m, Kpad);
                    tc::k_tc_gemm_tf32<<<dim3(Npad / 128, Upad / 128), tc::THREADS, tc::SMEM_BYTES, st>>>(
                        ma, mb, Cm, Npad, Kpad / tc::BK, err);
                    for (int ci = 0; ci < ncomp; ci++) {
                        double2 *o = acc + ((size_t)m * 6 + cs[ci]->vec * 3 + cs[ci]->axis) * ndir;
                        k_ff_reduce_tc<<<(ndir + 7) / 8, 256, 0, st>>>(o, Cm, Npad, ci * 2 * A, d_umap, d_r[F.a_ax],
                                                             d_r[F.n_ax], ndir, A, k, a_off, h[F.a_ax],
                                                             kind == 0, n0, area);
                    }
                }
                // this kind's operands go back to the stream-ordered pool for the next face
                for (void *q : {(void *)Am, (void *)Bm, (void *)Cm}) {
                    ck(cudaFreeAsync(q, st), "cudaFreeAsync");
                    tmp.erase(std::find(tmp.begin(), tmp.end(), q));
                }
                continue;
            }
            double2 *Pm = (double2 *)dmalloc((size_t)U * B * sizeof(double2));
            double2 *T = (double2 *)dmalloc((size_t)U * A * sizeof(double2));
            for (int m = 0; m < nf; m++) {
                const double k = 2 * kPI * P.fntf[m] / vp;
                k_ff_phase<<<dim3((B + 127) / 128, U), 128, 0, st>>>(Pm, d_s, U, B, k, b_off, h[F.b_ax],
                                                                     kind == 1);
                for (int c = 0; c < 4; c++) {
                    const CompDesc &C = kComps[F.n_ax][c];
                    if (C.kind != kind) continue;
                    const double *src = ntf[f * 4 + C.q];
                    k_ff_gemm<<<dim3((A + FT - 1) / FT, (U + FT - 1) / FT), dim3(FT, FT), 0, st>>>(
                        T, Pm, src, U, A, B, ntfb, ntfb, Nb, n2, m);
                    double2 *o = acc + ((size_t)m * 6 + C.vec * 3 + C.axis) * ndir;
                    k_ff_reduce<<<ndir, 256, 0, st>>>(o, T, d_umap, d_r[F.a_ax], d_r[F.n_ax], ndir, A, k,
                                                      a_off, h[F.a_ax], kind == 0, n0, area);
                }
            }
        }
    }
    // sigma on the device: analysis/meteorNTF.m:311-332, generalised to (theta, phi)
    double *d_th = (double *)dmalloc(ndir * 8), *d_ph = (double *)dmalloc(ndir * 8);
    double *d_sig = (double *)dmalloc((size_t)nf * ndir * 3 * 8);
    ck(cudaMemcpyAsync(d_th, theta, ndir * 8, cudaMemcpyHostToDevice, st), "H2D");
    ck(cudaMemcpyAsync(d_ph, phi, ndir * 8, cudaMemcpyHostToDevice, st), "H2D");
    const double *Eydft = srcdft, *Ezdft = srcdft + 2 * nf;
    for (int m = 0; m < nf; m++) {
        const double k = 2 * kPI * P.fntf[m] / vp;
        const double ezr = Ezdft[2 * m + 1], ezi = Ezdft[2 * m];
        const double eyr = Eydft[2 * m + 1], eyi = Eydft[2 * m];
        const double Pinc = (ezr * ezr + ezi * ezi + eyr * eyr + eyi * eyi) / 2 / eta0;
        k_ff_sigma<<<(ndir + 127) / 128, 128, 0, st>>>(acc + (size_t)m * 6 * ndir, ndir, d_th, d_ph, ndir,
                                                       k * k / (8 * kPI * eta0) / Pinc, eta0,
                                                       d_sig + (size_t)m * ndir * 3);
    }
    unsigned int herr = 0;
    ck(cudaMemcpyAsync(out, d_sig, (size_t)nf * ndir * 3 * 8, cudaMemcpyDeviceToHost, st), "D2H");
    ck(cudaMemcpyAsync(&herr, err, 4, cudaMemcpyDeviceToHost, st), "D2H");
    for (void *p : tmp) ck(cudaFreeAsync(p, st), "cudaFreeAsync");
    ck(cudaStreamSynchronize(st), "far field");
    if (herr) throw Error(MFDTD_ETIMEOUT, "far field: a tensor-core GEMM wait ran out");
}

}  // namespace mfdtd

// ---------------------------------------------------------------------------
// Far-field projection without any device allocation.
//
// Some callers cannot allocate device memory while they run: a plugin whose
// host application owns every device allocation, a service that reserves all
// of its memory up front and forbids allocation on the request path, or code
// that must not call into the CUDA allocator at all.  This variant keeps its
// working memory in one file-scope device array instead, so it only needs the
// inputs and outputs the caller already holds.  Its limits, and the reasons:
//   * the array belongs to this file's CUDA module.  With lazy module loading
//     (the CUDA default since 12.2) the module, and with it the array, is
//     created on each device the first time the process uses a kernel or
//     symbol of this file there -- typically the first call of this entry
//     point -- and held until the process exits.  A caller whose request path
//     must not allocate makes one warm-up call per device at start-up (also
//     before any stream capture).  The array is small for that reason;
//   * every call uses the same array, so calls whose GPU work overlaps (on two
//     streams, or from two threads) race with each other; callers must
//     serialise them;
//   * directions are processed 256 at a time and each face may be at most
//     2048 cells along either of its in-plane axes, which bounds the array.
namespace mfdtd {
namespace {

constexpr int kStaticDirs = 256;      // directions per pass
constexpr int kStaticFace = 2048;     // max in-plane face extent (cells)

// The regions carve() takes from the array, in order, each rounded up to 256
// bytes: P and T (one row of kStaticFace phasors per direction), the L and N
// accumulators (6 complex values per direction), then per direction theta,
// phi, the three components of r_hat, the three sigma values, and the
// identity direction map.  The array's size is computed from the same list.
constexpr size_t kStaticRegions[] = {
    (size_t)kStaticDirs * kStaticFace * sizeof(double2),   // P
    (size_t)kStaticDirs * kStaticFace * sizeof(double2),   // T
    (size_t)kStaticDirs * 6 * sizeof(double2),             // L, N accumulators
    kStaticDirs * sizeof(double), kStaticDirs * sizeof(double),  // theta, phi
    kStaticDirs * sizeof(double), kStaticDirs * sizeof(double), kStaticDirs * sizeof(double),  // r_hat
    (size_t)kStaticDirs * 3 * sizeof(double),              // sigma and its two terms
    kStaticDirs * sizeof(int),                             // identity direction map
};
constexpr size_t round256(size_t b) { return (b + 255) / 256 * 256; }
constexpr size_t static_bytes() {
    size_t t = 0;
    for (size_t b : kStaticRegions) t += round256(b);
    return t;
}
constexpr size_t kStaticBytes = static_bytes();
__device__ __align__(256) unsigned char g_ff_scratch[kStaticBytes];

struct StaticScratch {
    double2 *P, *T, *acc;
    double *th, *ph, *r[3], *sig;
    int *umap;
};

StaticScratch carve(unsigned char *base) {
    StaticScratch sc;
    size_t off = 0;
    int region = 0;
    auto take = [&]() {
        unsigned char *p = base + off;
        off += round256(kStaticRegions[region++]);
        return p;
    };
    sc.P = (double2 *)take();
    sc.T = (double2 *)take();
    sc.acc = (double2 *)take();
    sc.th = (double *)take();
    sc.ph = (double *)take();
    for (int q = 0; q < 3; q++) sc.r[q] = (double *)take();
    sc.sig = (double *)take();
    sc.umap = (int *)take();
    if (off != kStaticBytes || region != (int)(sizeof kStaticRegions / sizeof kStaticRegions[0]))
        throw Error(MFDTD_EINVAL, "allocation-free far field: scratch layout mismatch");
    return sc;
}

// Device address of g_ff_scratch on the current device.  The host-side symbol
// is only a stand-in, never a device address, so the address is looked up
// with the device current -- on every call: a cached address would go stale
// when the context is torn down (cudaDeviceReset) and the module reloaded.
unsigned char *scratch_for_current_device() {
    void *addr = nullptr;
    ck(cudaGetSymbolAddress(&addr, g_ff_scratch), "cudaGetSymbolAddress");
    return (unsigned char *)addr;
}

__global__ void k_ff_dirs(const double *th, const double *ph, int n, double *rx, double *ry, double *rz,
                          int *umap) {
    const int d = blockIdx.x * blockDim.x + threadIdx.x;
    if (d >= n) return;
    double st, ct, sp, cp;
    sincos(th[d], &st, &ct);
    sincos(ph[d], &sp, &cp);
    rx[d] = st * cp;
    ry[d] = st * sp;
    rz[d] = ct;
    umap[d] = d;
}

// sigma and its two polarisation terms from the L, N accumulators of n directions.

}  // namespace
}  // namespace mfdtd

extern "C" int mfdtd_far_field_static(const double *const ntf_dev[24], int32_t Nx, int32_t Ny, int32_t Nz,
                                      int32_t ntfb, int32_t nntf, const double *fntf, double dx, double dy,
                                      double dz, const double *srcdft, int32_t ndir, const double *theta,
                                      const double *phi, double *out, void *stream) {
    using namespace mfdtd;
    try {
        if (!ntf_dev || !fntf || !srcdft || !theta || !phi || !out || ndir <= 0 || nntf <= 0)
            throw Error(MFDTD_EINVAL, "NULL argument or empty direction/frequency list");
        for (int q = 0; q < 24; q++)
            if (!ntf_dev[q]) throw Error(MFDTD_EINVAL, "NULL face array");
        if (ntfb < 0) throw Error(MFDTD_EINVAL, "ntfb < 0: the Huygens faces lie outside the grid");
        const int dims[3] = {Nx, Ny, Nz};
        for (int q = 0; q < 3; q++)
            if (dims[q] - 2 * ntfb + 1 > kStaticFace || dims[q] - 2 * ntfb < 1)
                throw Error(MFDTD_EINVAL, "face extent outside [1, 2048] cells: too large for the "
                                          "allocation-free far field (use mfdtd_sim_far_field)");
        cudaStream_t st = (cudaStream_t)stream;
        const StaticScratch sc = carve(scratch_for_current_device());
        const double h[3] = {dx, dy, dz};
        const int n2 = 2 * nntf;
        const double vp = std::sqrt(1.0 / (kU0a * kE0a)), eta0 = std::sqrt(kU0a / kE0a);
        for (int d0 = 0; d0 < ndir; d0 += kStaticDirs) {
            const int nd = std::min(kStaticDirs, ndir - d0);
            ck(cudaMemcpyAsync(sc.th, theta + d0, nd * sizeof(double), cudaMemcpyHostToDevice, st), "H2D");
            ck(cudaMemcpyAsync(sc.ph, phi + d0, nd * sizeof(double), cudaMemcpyHostToDevice, st), "H2D");
            k_ff_dirs<<<(nd + 127) / 128, 128, 0, st>>>(sc.th, sc.ph, nd, sc.r[0], sc.r[1], sc.r[2], sc.umap);
            for (int m = 0; m < nntf; m++) {
                ck(cudaMemsetAsync(sc.acc, 0, (size_t)kStaticDirs * 6 * sizeof(double2), st), "memset");
                const double k = 2 * kPI * fntf[m] / vp;
                for (int f = 0; f < 6; f++) {
                    const FaceDesc &F = kFaces[f];
                    const int Na = dims[F.a_ax], Nb = dims[F.b_ax];
                    const double n0 = (F.high ? dims[F.n_ax] - ntfb : ntfb) * h[F.n_ax];
                    const double area = h[F.a_ax] * h[F.b_ax];
                    for (int kind = 0; kind < 2; kind++) {
                        const int A = kind == 0 ? Na - 2 * ntfb + 1 : Na - 2 * ntfb;
                        const int B = kind == 0 ? Nb - 2 * ntfb : Nb - 2 * ntfb + 1;
                        const double a_off = kind == 0 ? ntfb : ntfb + 0.5;
                        const double b_off = kind == 0 ? ntfb + 0.5 : ntfb;
                        // one P row per direction: P[d][b] = w_b exp(-jk r_b(d) pos_b)
                        k_ff_phase<<<dim3((B + 127) / 128, nd), 128, 0, st>>>(sc.P, sc.r[F.b_ax], nd, B, k, b_off,
                                                                              h[F.b_ax], kind == 1);
                        for (int c = 0; c < 4; c++) {
                            const CompDesc &C = kComps[F.n_ax][c];
                            if (C.kind != kind) continue;
                            k_ff_gemm<<<dim3((A + FT - 1) / FT, (nd + FT - 1) / FT), dim3(FT, FT), 0, st>>>(
                                sc.T, sc.P, ntf_dev[f * 4 + C.q], nd, A, B, ntfb, ntfb, Nb, n2, m);
                            k_ff_reduce<<<nd, 256, 0, st>>>(sc.acc + (size_t)(C.vec * 3 + C.axis) * kStaticDirs,
                                                            sc.T, sc.umap, sc.r[F.a_ax], sc.r[F.n_ax], nd, A, k,
                                                            a_off, h[F.a_ax], kind == 0, n0, area);
                        }
                    }
                }
                const double ezr = srcdft[2 * nntf + 2 * m + 1], ezi = srcdft[2 * nntf + 2 * m];
                const double eyr = srcdft[2 * m + 1], eyi = srcdft[2 * m];
                const double Pinc = (ezr * ezr + ezi * ezi + eyr * eyr + eyi * eyi) / 2 / eta0;
                k_ff_sigma<<<(nd + 127) / 128, 128, 0, st>>>(sc.acc, kStaticDirs, sc.th, sc.ph, nd,
                                                             k * k / (8 * kPI * eta0) / Pinc, eta0, sc.sig);
                ck(cudaMemcpyAsync(out + ((size_t)m * ndir + d0) * 3, sc.sig, (size_t)nd * 3 * sizeof(double),
                                   cudaMemcpyDeviceToHost, st),
                   "D2H");
            }
        }
        ck(cudaGetLastError(), "kernel launch");
        ck(cudaStreamSynchronize(st), "far field (static scratch)");
        return MFDTD_OK;
    } catch (const Error &e) {
        set_last_error(e.what());
        return e.code;
    } catch (const std::exception &e) {
        set_last_error(e.what());
        return MFDTD_EINVAL;
    }
}
