// bk_helmholtz.cu -- batched mixed-order Helmholtz operator and its CG solver.
//
// A plan describes elements of several orders p (2..8; BK5 points q = p + 1)
// stored one order after another (u, v, mass: E_p q^3 values each; G: E_p 6
// q^3 values in the column layout), cut into tiles whose sizes per order
// come from the caller (the autotuner of omp_bk_gb300.tune).  The apply
// v = D^T G D u + lambda mass u is ONE persistent launch over the tile list
// (bk5_multi.cuh): the even-odd sweep body when every D is
// centro-antisymmetric (GLL), the column body otherwise or on request.
//
// The solver is conjugate gradients in mixed precision with FP64 residual
// refinement: the outer loop forms the FP64 residual r = f - A x with the
// FP64-accurate apply (float-float engine, FP64 storage) and stops at
// |r| <= rtol |f|; the inner loop solves A d = r / |r| approximately with CG
// on the FP32-storage operator (mixed engine), FP32 vectors and FP64 dot
// products, and x += |r| d.  The inner CG is captured once in a CUDA graph:
// its iteration (apply, dot, updates, next direction) is the body of a
// conditional WHILE node whose condition a device kernel sets from the
// residual, so the whole inner solve is one graph launch with no host round
// trip.  The reference has no solver; this is the standard preconditioner-free
// CG (Hestenes-Stiefel) with iterative refinement.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include <cuda_runtime.h>

#include "bk5_multi.cuh"
#include "bk_internal.h"
#include "bk_solver.h"

namespace bkg {
namespace {

constexpr int kNT = 256;   // threads per block of the persistent kernel (per thread group), at most
constexpr int kMaxTileLines = 1024;   // lines (elements x q^2) of a tile, at most
constexpr int kRedBlocks = 1216;   // 8 blocks of 256 threads per SM
constexpr int kMaxDotParts = 4864;  // blocks of the persistent launch at most (32 per SM)
constexpr int kRedThreads = 256;

enum Scalar { S_RR = 0, S_RR0, S_PAP, S_IT, S_TOL2, S_MAXIT, S_NORM, S_INV, S_RN2, S_FN2, S_NSCAL };

template <class Eng, int NBUF>
struct MultiLaunch {
    // Sets the kernel's shared-memory limit on the current device (once) and
    // returns its resident blocks per SM for `total` bytes; outside any
    // stream capture.
    static int prepare(int total)
    {
        auto kern = bk5_multi_kernel<Eng, kNT, NBUF>;
        static int set[kMaxDevices] = {0};
        static int occ_of[kMaxDevices][2] = {{0, 0}};
        const int dev = current_device();
        if (dev < 0 || dev >= kMaxDevices) return 0;
        if (!set[dev]) {
            if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, 232448) != cudaSuccess) {
                cudaGetLastError();
                return 0;
            }
            set[dev] = 1;
        }
        if (occ_of[dev][0] != total) {
            int occ = 0;
            if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, kNT, total) != cudaSuccess) {
                cudaGetLastError();
                return 0;
            }
            occ_of[dev][0] = total;
            occ_of[dev][1] = occ;
        }
        return occ_of[dev][1];
    }

    static int smem(const PMulti<typename Eng::C>& prm, int& st, int& cb)
    {
        int total = 0;
        multi_smem<Eng>(prm.seg, prm.nseg, st, cb, total, NBUF);
        return total;
    }

    static int run(const PMulti<typename Eng::C>& prm, const MultiTile* tiles, int ntiles, const void* u,
                   const void* G, const void* mass, double lambda, void* v, cudaStream_t s)
    {
        using S = typename Eng::S;
        int st = 0, cb = 0;
        const int total = smem(prm, st, cb);
        if (total > 232448) return BK_ERR_ARG;
        auto kern = bk5_multi_kernel<Eng, kNT, NBUF>;
        const int occ = prepare(total);
        if (occ < 1) return BK_ERR_CUDA;
        int grid = occ * sm_count();
        if (grid > ntiles) grid = ntiles;
        if (grid < 1) return BK_OK;
        kern<<<grid, kNT, total, s>>>(prm, tiles, ntiles, static_cast<const S*>(u), static_cast<const S*>(G),
                                      static_cast<const S*>(mass), lambda, static_cast<S*>(v), st, cb, dev_ctx());
        return cudaGetLastError() == cudaSuccess ? BK_OK : BK_ERR_CUDA;
    }
};

// The even-odd sweep launch: blockDim = the largest tile's lines (eb q^2),
// rounded up to whole warps, or the plan's block size when that is smaller
// (the sweeps of a tile with more lines than threads loop over them); three
// times that with direction-parallel groups (DPAR); MAXT threads at most,
// MINB blocks per SM asked of the register allocator.  GST: FP32 G staged.
template <class Eng, int MAXT, int MINB, bool DOT = false, int DPAR = 0, bool GST = false>
struct MultiEOLaunch {
    static int threads(const MultiSeg* seg, int nseg, int block)
    {
        int nt = 64;
        for (int s = 0; s < nseg; ++s) {
            const int l = (seg[s].eb * seg[s].q * seg[s].q + 31) / 32 * 32;
            nt = l > nt ? l : nt;
        }
        if (block > 0 && nt > block) nt = block;
        if (DPAR) nt *= 3;
        return nt > MAXT ? MAXT : nt;
    }
    static int smem(const PMultiEO<typename Eng::C>& prm, int& ub, int& gb, int& wb)
    {
        int total = 0;
        multi_eo_smem<Eng>(prm.seg, prm.nseg, ub, gb, wb, total, DPAR, GST);
        return total;
    }
    static int prepare(int total, int nt)
    {
        auto kern = bk5_multi_eo_kernel<Eng, MAXT, MINB, DOT, DPAR, GST>;
        static int set[kMaxDevices] = {0};
        static int occ_of[kMaxDevices][3] = {{0, 0, 0}};
        const int dev = current_device();
        if (dev < 0 || dev >= kMaxDevices) return 0;
        if (!set[dev]) {
            if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, 232448) != cudaSuccess) {
                cudaGetLastError();
                return 0;
            }
            set[dev] = 1;
        }
        if (occ_of[dev][0] != total || occ_of[dev][1] != nt) {
            int occ = 0;
            if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, nt, total) != cudaSuccess) {
                cudaGetLastError();
                return 0;
            }
            occ_of[dev][0] = total;
            occ_of[dev][1] = nt;
            occ_of[dev][2] = occ;
        }
        return occ_of[dev][2];
    }
    static int prepare(const PMultiEO<typename Eng::C>& prm)
    {
        int ub = 0, gb = 0, wb = 0;
        const int total = smem(prm, ub, gb, wb);
        if (total > 232448) return 0;
        return prepare(total, threads(prm.seg, prm.nseg, prm.block));
    }
    // dot_part (optional): one partial sum of u . v per block, their count in
    // *nparts
    static int run(const PMultiEO<typename Eng::C>& prm, const MultiTile* tiles, int ntiles, const void* u,
                   const void* G, const void* mass, double lambda, void* v, cudaStream_t s,
                   double* dot_part = nullptr, int* nparts = nullptr)
    {
        using S = typename Eng::S;
        int ub = 0, gb = 0, wb = 0;
        const int total = smem(prm, ub, gb, wb);
        const int nt = threads(prm.seg, prm.nseg, prm.block);
        if (total > 232448) return BK_ERR_ARG;
        if (DOT != (dot_part != nullptr)) return BK_ERR_ARG;
        auto kern = bk5_multi_eo_kernel<Eng, MAXT, MINB, DOT, DPAR, GST>;
        const int occ = prepare(total, nt);
        if (occ < 1) return BK_ERR_CUDA;
        int grid = occ * sm_count();
        if (grid > ntiles) grid = ntiles;
        if (grid > kMaxDotParts) grid = kMaxDotParts;
        if (nparts) *nparts = grid;
        if (grid < 1) return BK_OK;
        kern<<<grid, nt, total, s>>>(prm, tiles, ntiles, static_cast<const S*>(u), static_cast<const S*>(G),
                                     static_cast<const S*>(mass), lambda, static_cast<S*>(v), ub, gb, wb, dot_part,
                                     dev_ctx());
        return cudaGetLastError() == cudaSuccess ? BK_OK : BK_ERR_CUDA;
    }
};

// The float-float (FP64) launch: direction-parallel groups, three per block
// of up to 3 x 256 threads (the groups' shared body needs few registers).
using MultiFF = MultiEOLaunch<EngFF, 768, 1, false, 2>;

// The FP32-storage launches with G read from global memory or staged (the
// plan's gstage), with and without the fused dot product.
template <class Eng, bool DOT = false>
int run_f32(const PMultiEO<float>& prm, const MultiTile* tiles, int ntiles, const void* u, const void* G,
            const void* mass, double lambda, void* v, cudaStream_t s, double* dot_part = nullptr, int* nparts = nullptr)
{
    if (prm.gstage)
        return MultiEOLaunch<Eng, 256, 4, DOT, 0, true>::run(prm, tiles, ntiles, u, G, mass, lambda, v, s, dot_part,
                                                             nparts);
    return MultiEOLaunch<Eng, 256, 4, DOT, 0, false>::run(prm, tiles, ntiles, u, G, mass, lambda, v, s, dot_part,
                                                          nparts);
}

template <class Eng, bool DOT = false>
int prepare_f32(const PMultiEO<float>& prm)
{
    return prm.gstage ? MultiEOLaunch<Eng, 256, 4, DOT, 0, true>::prepare(prm)
                      : MultiEOLaunch<Eng, 256, 4, DOT, 0, false>::prepare(prm);
}

template <class Eng>
int smem_f32(const PMultiEO<float>& prm)
{
    int ub = 0, gb = 0, wb = 0;
    return prm.gstage ? MultiEOLaunch<Eng, 256, 4, false, 0, true>::smem(prm, ub, gb, wb)
                      : MultiEOLaunch<Eng, 256, 4, false, 0, false>::smem(prm, ub, gb, wb);
}

// ---- CG kernels --------------------------------------------------------------

// The diagonal of A = D^T G D + lambda M at the points of segment s (FP64
// from the stored G and mass): with e_x the unit vector of point x = (i, j,
// k), (D_r e_x)(y) = D(y_i, i) on the line through x along i and zero
// elsewhere, so the three directions' own terms are sums along the lines
// through x and the mixed terms meet only at x:
//   A_xx = sum_n D(n,i)^2 G_rr(n,j,k) + D(n,j)^2 G_ss(i,n,k) + D(n,k)^2 G_tt(i,j,n)
//        + 2 (D(i,i) D(j,j) G_rs + D(i,i) D(k,k) G_rt + D(j,j) D(k,k) G_st)(x)
//        + lambda mass(x).
// G in the column layout G(e, f, k, i, j).  out: A_xx (double) or its
// inverse (float, the Jacobi preconditioner of the inner CG).
template <class T, class O, bool INV>
__global__ void diag_kernel(const __grid_constant__ PMulti<double> prm, int s, const T* __restrict__ G,
                            const T* __restrict__ mass, double lambda, O* __restrict__ out)
{
    const MultiSeg sg = prm.seg[s];
    const int q = sg.q, q2 = q * q, q3 = q2 * q;
    const double* Dq = prm.D + multi_doff(q);   // D(a, b) = Dq[a*q + b]
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < sg.E * q3;
         t += (long long)gridDim.x * blockDim.x) {
        const long long e = t / q3;
        const int x = int(t - e * q3);
        const int i = x / q2, j = (x / q) % q, k = x % q;
        const T* Ge = G + sg.goff + e * 6 * q3;
        auto g = [&](int f, int a, int b, int c) { return double(Ge[((f * q + c) * q + a) * q + b]); };   // (i,j,k) = (a,b,c)
        double acc = 0.0;
        for (int n = 0; n < q; ++n) {
            const double di = Dq[n * q + i], dj = Dq[n * q + j], dk = Dq[n * q + k];
            acc += di * di * g(0, n, j, k) + dj * dj * g(3, i, n, k) + dk * dk * g(5, i, j, n);
        }
        const double dii = Dq[i * q + i], djj = Dq[j * q + j], dkk = Dq[k * q + k];
        acc += 2.0 * (dii * djj * g(1, i, j, k) + dii * dkk * g(2, i, j, k) + djj * dkk * g(4, i, j, k));
        if (mass != nullptr) acc += lambda * double(mass[sg.uoff + t]);
        if constexpr (INV)
            out[sg.uoff + t] = O(acc != 0.0 ? 1.0 / acc : 1.0);
        else
            out[sg.uoff + t] = O(acc);
    }
}

__global__ void fill_ones_kernel(long long n, float* __restrict__ x)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        x[i] = 1.0f;
}

// r = r64 / |r|, d = 0, p = z = invd .* r (Jacobi; invd = 1 without it)
__global__ void cg_start_kernel(long long n, const double* __restrict__ r64, const double* __restrict__ sc,
                                const float* __restrict__ invd, float* __restrict__ r, float* __restrict__ p,
                                float* __restrict__ d)
{
    const double inv = sc[S_INV];
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float x = float(r64[i] * inv);
        r[i] = x;
        p[i] = invd[i] * x;
        d[i] = 0.0f;
    }
}

// The FP32 vectors of the inner CG are 16-byte aligned allocations: their
// loops run over float4 groups (one 16-byte load per vector and thread and
// iteration, enough bytes in flight for HBM) and a scalar tail of n % 4.

__device__ __forceinline__ double block_reduce(double s)
{
    __shared__ double sh[kRedThreads];
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int w = kRedThreads / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
        __syncthreads();
    }
    return sh[0];
}

// partial sums of x.y (FP64) per block
__global__ void __launch_bounds__(kRedThreads) red_dot_kernel(long long n, const float* __restrict__ x,
                                                              const float* __restrict__ y, double* __restrict__ part)
{
    const long long n4 = n / 4;
    const long long stride = (long long)gridDim.x * kRedThreads;
    const float4* x4 = reinterpret_cast<const float4*>(x);
    const float4* y4 = reinterpret_cast<const float4*>(y);
    double s = 0.0;
    for (long long i = blockIdx.x * (long long)kRedThreads + threadIdx.x; i < n4; i += stride) {
        const float4 a = x4[i], b = y4[i];
        s = fma(double(a.x), double(b.x), s);
        s = fma(double(a.y), double(b.y), s);
        s = fma(double(a.z), double(b.z), s);
        s = fma(double(a.w), double(b.w), s);
    }
    for (long long i = 4 * n4 + blockIdx.x * (long long)kRedThreads + threadIdx.x; i < n; i += stride)
        s = fma(double(x[i]), double(y[i]), s);
    const double t = block_reduce(s);
    if (threadIdx.x == 0) part[blockIdx.x] = t;
}

__device__ __forceinline__ double block_sum(const double* __restrict__ part, int nb)
{
    __shared__ double sh[kRedThreads];
    double s = 0.0;
    for (int i = threadIdx.x; i < nb; i += kRedThreads) s += part[i];
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int w = kRedThreads / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
        __syncthreads();
    }
    return sh[0];
}

// scalars after the first r.r: rr0 = rr, it = 0
__global__ void __launch_bounds__(kRedThreads) cg_init_scalars_kernel(const double* __restrict__ part, int nb,
                                                                      double* __restrict__ sc)
{
    const double rr = block_sum(part, nb);
    if (threadIdx.x == 0) {
        sc[S_RR] = rr;
        sc[S_RR0] = rr;
        sc[S_IT] = 0.0;
    }
}

__global__ void __launch_bounds__(kRedThreads) cg_pap_kernel(const double* __restrict__ part, int nb,
                                                             double* __restrict__ sc)
{
    const double pap = block_sum(part, nb);
    if (threadIdx.x == 0) sc[S_PAP] = pap;
}

// d += alpha p, r -= alpha Ap and the partial sums of r.z = r.(invd .* r)
// (the preconditioned CG's r.z; r.r without the preconditioner, invd = 1)
__global__ void __launch_bounds__(kRedThreads) cg_update_kernel(long long n, const double* __restrict__ sc,
                                                                const float* __restrict__ p,
                                                                const float* __restrict__ Ap, float* __restrict__ d,
                                                                float* __restrict__ r, const float* __restrict__ invd,
                                                                double* __restrict__ part)
{
    const double pap = sc[S_PAP];
    const float alpha = float(pap != 0.0 ? sc[S_RR] / pap : 0.0);
    const long long n4 = n / 4;
    const long long stride = (long long)gridDim.x * kRedThreads;
    double s = 0.0;
    for (long long i = blockIdx.x * (long long)kRedThreads + threadIdx.x; i < n4; i += stride) {
        const float4 pp = reinterpret_cast<const float4*>(p)[i];
        const float4 aa = reinterpret_cast<const float4*>(Ap)[i];
        float4 dd = reinterpret_cast<float4*>(d)[i];
        float4 rr = reinterpret_cast<float4*>(r)[i];
        dd.x = fmaf(alpha, pp.x, dd.x);
        dd.y = fmaf(alpha, pp.y, dd.y);
        dd.z = fmaf(alpha, pp.z, dd.z);
        dd.w = fmaf(alpha, pp.w, dd.w);
        rr.x = fmaf(-alpha, aa.x, rr.x);
        rr.y = fmaf(-alpha, aa.y, rr.y);
        rr.z = fmaf(-alpha, aa.z, rr.z);
        rr.w = fmaf(-alpha, aa.w, rr.w);
        reinterpret_cast<float4*>(d)[i] = dd;
        reinterpret_cast<float4*>(r)[i] = rr;
        const float4 w = reinterpret_cast<const float4*>(invd)[i];
        s = fma(double(rr.x), double(w.x * rr.x), s);
        s = fma(double(rr.y), double(w.y * rr.y), s);
        s = fma(double(rr.z), double(w.z * rr.z), s);
        s = fma(double(rr.w), double(w.w * rr.w), s);
    }
    for (long long i = 4 * n4 + blockIdx.x * (long long)kRedThreads + threadIdx.x; i < n; i += stride) {
        d[i] = fmaf(alpha, p[i], d[i]);
        const float ri = fmaf(-alpha, Ap[i], r[i]);
        r[i] = ri;
        s = fma(double(ri), double(invd[i] * ri), s);
    }
    const double t = block_reduce(s);
    if (threadIdx.x == 0) part[blockIdx.x] = t;
}

// rr_new, beta, iteration count and the loop condition
__global__ void __launch_bounds__(kRedThreads) cg_step_kernel(const double* __restrict__ part, int nb,
                                                              double* __restrict__ sc, double* __restrict__ beta_out,
                                                              cudaGraphConditionalHandle handle)
{
    const double rr = block_sum(part, nb);
    if (threadIdx.x == 0) {
        const double old = sc[S_RR];
        beta_out[0] = old != 0.0 ? rr / old : 0.0;
        sc[S_RR] = rr;
        const double it = sc[S_IT] + 1.0;
        sc[S_IT] = it;
        const bool go = (rr > sc[S_TOL2] * sc[S_RR0]) && (it < sc[S_MAXIT]);
        cudaGraphSetConditional(handle, go ? 1u : 0u);
    }
}

// p = z + beta p, z = invd .* r
__global__ void cg_dir_kernel(long long n, const double* __restrict__ beta_in, const float* __restrict__ r,
                              const float* __restrict__ invd, float* __restrict__ p)
{
    const float beta = float(beta_in[0]);
    const long long n4 = n / 4;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n4; i += stride) {
        const float4 rr = reinterpret_cast<const float4*>(r)[i];
        const float4 w = reinterpret_cast<const float4*>(invd)[i];
        float4 pp = reinterpret_cast<float4*>(p)[i];
        pp.x = fmaf(beta, pp.x, w.x * rr.x);
        pp.y = fmaf(beta, pp.y, w.y * rr.y);
        pp.z = fmaf(beta, pp.z, w.z * rr.z);
        pp.w = fmaf(beta, pp.w, w.w * rr.w);
        reinterpret_cast<float4*>(p)[i] = pp;
    }
    for (long long i = 4 * n4 + blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += stride)
        p[i] = fmaf(beta, p[i], invd[i] * r[i]);
}
// x += |r| d (FP64), the norm from the scalars
__global__ void cg_correct_kernel(long long n, const double* __restrict__ sc, const float* __restrict__ d,
                                  double* __restrict__ x)
{
    const double nrm = sc[S_NORM];
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        x[i] = fma(nrm, double(d[i]), x[i]);
}

// r = f - r (the apply wrote A x into r); partial sums of r.r
__global__ void __launch_bounds__(kRedThreads) res64_kernel(long long n, const double* __restrict__ f,
                                                            double* __restrict__ r, double* __restrict__ part)
{
    __shared__ double sh[kRedThreads];
    double s = 0.0;
    for (long long i = blockIdx.x * (long long)kRedThreads + threadIdx.x; i < n; i += (long long)gridDim.x * kRedThreads) {
        const double ri = f[i] - r[i];
        r[i] = ri;
        s = fma(ri, ri, s);
    }
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int w = kRedThreads / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}

__global__ void __launch_bounds__(kRedThreads) norm_kernel(const double* __restrict__ part, int nb,
                                                           double* __restrict__ sc)
{
    const double rn2 = block_sum(part, nb);
    if (threadIdx.x == 0) {
        sc[S_RN2] = rn2;
        const double nrm = sqrt(rn2);
        sc[S_NORM] = nrm;
        sc[S_INV] = nrm > 0.0 ? 1.0 / nrm : 0.0;
    }
}

__global__ void __launch_bounds__(kRedThreads) dot64_partial_kernel(long long n, const double* __restrict__ x,
                                                                    const double* __restrict__ y,
                                                                    double* __restrict__ part)
{
    __shared__ double sh[kRedThreads];
    double s = 0.0;
    for (long long i = blockIdx.x * (long long)kRedThreads + threadIdx.x; i < n; i += (long long)gridDim.x * kRedThreads)
        s = fma(x[i], y[i], s);
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int w = kRedThreads / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}

__global__ void __launch_bounds__(kRedThreads) sum_to_kernel(const double* __restrict__ part, int nb,
                                                             double* __restrict__ out)
{
    const double v = block_sum(part, nb);
    if (threadIdx.x == 0) out[0] = v;
}

int grid_n(long long n)
{
    const long long g = (n + 1023) / 1024;
    return int(g < 1216 ? (g > 0 ? g : 1) : 1216);
}

}  // namespace
}  // namespace bkg

using namespace bkg;

struct bk_hplan {
    int device;
    int nseg;
    MultiSeg seg[kMultiNQ];
    std::vector<MultiTile> htiles;
    MultiTile* tiles;   // device
    int ntiles;
    // the FP64-storage sweep launches' own tiles (bk_hplan_set_fp64_shape;
    // NULL: the plan's tiles)
    MultiTile* tiles64;
    int ntiles64;
    long long n;        // values of a vector
    long long ng;       // values of G
    PMulti<double> p_dfma;
    PMulti<ff> p_ff;
    PMulti<float> p_f32;
    // the even-odd forms (valid when eo_ok)
    PMultiEO<double> e_dfma;
    PMultiEO<ff> e_ff;
    PMultiEO<float> e_f32;
    bool eo_ok;
    int kernel;         // BK_KERNEL_SWEEP (even-odd) or BK_KERNEL_COLUMN
    // solver state
    double* r64;
    float* r32;
    float* p32;
    float* Ap32;
    float* d32;
    float* invd;        // the inner CG's Jacobi preconditioner (ones without it)
    double* part;
    double* sc;
    double* beta;
    cudaGraphExec_t inner_exec;
    cudaGraph_t inner_graph;
    const void* g_key[3];   // operator pointers the graph was built for
    double key_lambda;
    int key_precond;
};

namespace {

template <class C>
void fill_params(PMulti<C>& P, const bk_hplan& h, const double* const* Dq, C (*conv)(double))
{
    std::memset(&P, 0, sizeof(P));
    for (int s = 0; s < h.nseg; ++s) {
        const int q = h.seg[s].q;
        for (int x = 0; x < q * q; ++x) P.D[multi_doff(q) + x] = conv(Dq[s][x]);
        P.seg[s] = h.seg[s];
    }
    P.nseg = h.nseg;
    P.n = h.n;
    P.ng = h.ng;
}

template <class C, class Conv>
bool fill_eo_params(PMultiEO<C>& P, const bk_hplan& h, const double* const* Dq, Conv conv)
{
    std::memset(&P, 0, sizeof(P));
    bool ok = true;
    for (int s = 0; s < h.nseg; ++s) {
        ok = multi_eo_fill(P.eo, h.seg[s].q, Dq[s], conv) && ok;
        P.seg[s] = h.seg[s];
    }
    P.nseg = h.nseg;
    P.n = h.n;
    P.ng = h.ng;
    return ok;
}

// The tile list of segments seg[0, nseg): tiles of seg[s].eb elements, the
// most expensive order first.
std::vector<MultiTile> make_tiles(const MultiSeg* seg, int nseg)
{
    std::vector<int> order(nseg);
    for (int s = 0; s < nseg; ++s) order[s] = s;
    for (int a = 0; a < nseg; ++a)
        for (int b = a + 1; b < nseg; ++b)
            if (seg[order[b]].q > seg[order[a]].q) std::swap(order[a], order[b]);
    std::vector<MultiTile> t;
    for (int s : order) {
        for (long long e = 0; e < seg[s].E; e += seg[s].eb) {
            MultiTile x;
            x.seg = s;
            x.ne = int((seg[s].E - e) < seg[s].eb ? (seg[s].E - e) : seg[s].eb);
            x.e_first = e;
            t.push_back(x);
        }
    }
    return t;
}

double conv_d(double x) { return x; }
float conv_f(double x) { return float(x); }
ff conv_ff(double x) { return EngFF::coef(x); }

int apply_plan(bk_hplan* h, int eng, const void* G, const void* mass, double lambda, const void* u, void* v,
               cudaStream_t s)
{
    if (h->kernel == BK_KERNEL_SWEEP) {
        const MultiTile* t64 = h->tiles64 ? h->tiles64 : h->tiles;
        const int n64 = h->tiles64 ? h->ntiles64 : h->ntiles;
        switch (eng) {
            case 0: return MultiEOLaunch<EngDfma, 256, 2>::run(h->e_dfma, t64, n64, u, G, mass, lambda, v, s);
            case 1: return MultiFF::run(h->e_ff, t64, n64, u, G, mass, lambda, v, s);
            case 2: return run_f32<EngF32>(h->e_f32, h->tiles, h->ntiles, u, G, mass, lambda, v, s);
            default:
                return run_f32<EngMixed>(h->e_f32, h->tiles, h->ntiles, u, G, mass, lambda, v, s);
        }
    }
    switch (eng) {
        case 0: return MultiLaunch<EngDfma, 1>::run(h->p_dfma, h->tiles, h->ntiles, u, G, mass, lambda, v, s);
        case 1: return MultiLaunch<EngFF, 1>::run(h->p_ff, h->tiles, h->ntiles, u, G, mass, lambda, v, s);
        case 2: return MultiLaunch<EngF32, 2>::run(h->p_f32, h->tiles, h->ntiles, u, G, mass, lambda, v, s);
        default: return MultiLaunch<EngMixed, 2>::run(h->p_f32, h->tiles, h->ntiles, u, G, mass, lambda, v, s);
    }
}

int ck(cudaError_t e) { return e == cudaSuccess ? BK_OK : BK_ERR_CUDA; }

// The column body has one thread per k-column of a tile: every tile's
// columns (elements x q^2) must fit one block.
bool column_fits(const bk_hplan& h)
{
    for (int s = 0; s < h.nseg; ++s)
        if (h.seg[s].eb * h.seg[s].q * h.seg[s].q > kNT) return false;
    return true;
}

void free_graph(bk_hplan* h)
{
    if (h->inner_exec) cudaGraphExecDestroy(h->inner_exec);
    if (h->inner_graph) cudaGraphDestroy(h->inner_graph);
    h->inner_exec = nullptr;
    h->inner_graph = nullptr;
}

// The inner CG as a graph: start, r.r, then WHILE(cond) { A p, p.Ap, update,
// step (sets cond), new direction }.
// invd = 1 / diag(A) from the FP32 operator (precond), or ones.
int fill_precond(bk_hplan* h, const void* G32, const void* mass32, double lambda, int precond, cudaStream_t s)
{
    if (!precond) {
        fill_ones_kernel<<<grid_n(h->n), 256, 0, s>>>(h->n, h->invd);
        return ck(cudaGetLastError());
    }
    for (int sg = 0; sg < h->nseg; ++sg) {
        const long long np = h->seg[sg].E * h->seg[sg].q * h->seg[sg].q * h->seg[sg].q;
        if (np == 0) continue;
        diag_kernel<float, float, true><<<grid_n(np), 256, 0, s>>>(h->p_dfma, sg, static_cast<const float*>(G32),
                                                                   static_cast<const float*>(mass32), lambda, h->invd);
    }
    return ck(cudaGetLastError());
}

int build_inner_graph(bk_hplan* h, const void* G32, const void* mass32, double lambda, int precond, cudaStream_t user)
{
    free_graph(h);
    {
        // kernel attributes and occupancy outside the capture
        int st = 0, cb = 0;
        if (h->kernel == BK_KERNEL_SWEEP) {
            if (prepare_f32<EngMixed, true>(h->e_f32) < 1) return BK_ERR_CUDA;
        } else if (MultiLaunch<EngMixed, 2>::prepare(MultiLaunch<EngMixed, 2>::smem(h->p_f32, st, cb)) < 1) {
            return BK_ERR_CUDA;
        }
    }
    // the legacy default stream cannot be captured: capture on a private
    // stream (the graph is launched on the caller's stream)
    (void)user;
    cudaStream_t s = nullptr;
    if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) {
        cudaGetLastError();
        return BK_ERR_CUDA;
    }
    struct StreamGuard {
        cudaStream_t s;
        ~StreamGuard() { cudaStreamDestroy(s); }
    } guard{s};
    cudaGraph_t g = nullptr;
    if (cudaGraphCreate(&g, 0) != cudaSuccess) {
        cudaGetLastError();
        return BK_ERR_CUDA;
    }
    cudaGraphConditionalHandle handle;
    if (cudaGraphConditionalHandleCreate(&handle, g, 1, cudaGraphCondAssignDefault) != cudaSuccess) {
        cudaGetLastError();
        cudaGraphDestroy(g);
        return BK_ERR_CUDA;
    }
    const long long n = h->n;
    const int gn = grid_n(n);
    // prologue, captured into g
    int rc = BK_OK;
    if (cudaStreamBeginCaptureToGraph(s, g, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
        cudaGetLastError();
        cudaGraphDestroy(g);
        return BK_ERR_CUDA;
    }
    cg_start_kernel<<<gn, 256, 0, s>>>(n, h->r64, h->sc, h->invd, h->r32, h->p32, h->d32);
    red_dot_kernel<<<kRedBlocks, kRedThreads, 0, s>>>(n, h->r32, h->p32, h->part);   // r.z
    cg_init_scalars_kernel<<<1, kRedThreads, 0, s>>>(h->part, kRedBlocks, h->sc);
    cudaGraph_t captured = nullptr;
    if (cudaStreamEndCapture(s, &captured) != cudaSuccess) rc = BK_ERR_CUDA;
    // the WHILE node after the prologue
    cudaGraphNode_t leaf = nullptr;
    if (rc == BK_OK) {
        size_t nn = 0;
        cudaGraphGetNodes(g, nullptr, &nn);
        std::vector<cudaGraphNode_t> nodes(nn);
        cudaGraphGetNodes(g, nodes.data(), &nn);
        for (cudaGraphNode_t nd : nodes) {
            size_t ndep = 0;
            cudaGraphNodeGetDependentNodes(nd, nullptr, nullptr, &ndep);
            if (ndep == 0) leaf = nd;
        }
        cudaGraphNodeParams cp = {};
        cp.type = cudaGraphNodeTypeConditional;
        cp.conditional.handle = handle;
        cp.conditional.type = cudaGraphCondTypeWhile;
        cp.conditional.size = 1;
        cudaGraphNode_t cnode;
        if (cudaGraphAddNode(&cnode, g, leaf ? &leaf : nullptr, nullptr, leaf ? 1 : 0, &cp) != cudaSuccess) {
            rc = BK_ERR_CUDA;
        } else {
            cudaGraph_t body = cp.conditional.phGraph_out[0];
            if (cudaStreamBeginCaptureToGraph(s, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal) !=
                cudaSuccess) {
                rc = BK_ERR_CUDA;
            } else {
                int arc;
                if (h->kernel == BK_KERNEL_SWEEP) {
                    // p . Ap summed by the apply itself (one partial per block)
                    int nparts = 0;
                    arc = run_f32<EngMixed, true>(h->e_f32, h->tiles, h->ntiles, h->p32, G32, mass32, lambda, h->Ap32,
                                                  s, h->part, &nparts);
                    cg_pap_kernel<<<1, kRedThreads, 0, s>>>(h->part, nparts, h->sc);
                } else {
                    arc = apply_plan(h, 3, G32, mass32, lambda, h->p32, h->Ap32, s);
                    red_dot_kernel<<<kRedBlocks, kRedThreads, 0, s>>>(n, h->p32, h->Ap32, h->part);
                    cg_pap_kernel<<<1, kRedThreads, 0, s>>>(h->part, kRedBlocks, h->sc);
                }
                cg_update_kernel<<<kRedBlocks, kRedThreads, 0, s>>>(n, h->sc, h->p32, h->Ap32, h->d32, h->r32,
                                                                    h->invd, h->part);
                cg_step_kernel<<<1, kRedThreads, 0, s>>>(h->part, kRedBlocks, h->sc, h->beta, handle);
                cg_dir_kernel<<<gn, 256, 0, s>>>(n, h->beta, h->r32, h->invd, h->p32);
                cudaGraph_t body_out = nullptr;
                if (cudaStreamEndCapture(s, &body_out) != cudaSuccess || arc != BK_OK) rc = BK_ERR_CUDA;
            }
        }
    }
    if (rc == BK_OK && cudaGraphInstantiate(&h->inner_exec, g, 0) != cudaSuccess) rc = BK_ERR_CUDA;
    if (rc != BK_OK) {
        cudaGetLastError();
        cudaGraphDestroy(g);
        h->inner_exec = nullptr;
        return rc;
    }
    h->inner_graph = g;
    h->g_key[0] = G32;
    h->g_key[1] = mass32;
    h->key_lambda = lambda;
    h->key_precond = precond;
    return BK_OK;
}

}  // namespace

extern "C" {

int bk_hplan_create(bk_hplan_t* out, int norders, const bk_order_range* orders, const double* const* D,
                    bk_stream_t stream)
{
    if (!out || !orders || !D) return BK_ERR_NULL;
    *out = nullptr;
    if (norders < 1 || norders > kMultiNQ) return BK_ERR_ARG;
    bk_hplan* h = new bk_hplan();
    std::memset(h->seg, 0, sizeof(h->seg));
    h->device = current_device();
    h->nseg = norders;
    long long uo = 0, go = 0;
    for (int s = 0; s < norders; ++s) {
        const int p = orders[s].p;
        if (p < kMultiQmin - 1 || p > kMultiQmax - 1) {
            delete h;
            return BK_ERR_ORDER;
        }
        const int q = p + 1;
        int eb = orders[s].elems_per_tile;
        if (eb <= 0) eb = (q * q >= 100) ? 1 : ((q * q >= 64) ? 2 : (128 + q * q - 1) / (q * q));
        if (eb * q * q > kMaxTileLines || orders[s].E < 0 || !D[s]) {
            delete h;
            return orders[s].E < 0 ? BK_ERR_SIZE : BK_ERR_ARG;
        }
        h->seg[s].q = q;
        h->seg[s].eb = eb;
        h->seg[s].E = orders[s].E;
        h->seg[s].uoff = uo;
        h->seg[s].goff = go;
        uo += orders[s].E * q * q * q;
        go += orders[s].E * 6 * q * q * q;
    }
    h->n = uo;
    h->ng = go;
    h->htiles = make_tiles(h->seg, norders);
    h->ntiles = int(h->htiles.size());
    fill_params(h->p_dfma, *h, D, conv_d);
    fill_params(h->p_ff, *h, D, conv_ff);
    fill_params(h->p_f32, *h, D, conv_f);
    h->eo_ok = fill_eo_params(h->e_dfma, *h, D, conv_d) && fill_eo_params(h->e_ff, *h, D, conv_ff) &&
               fill_eo_params(h->e_f32, *h, D, conv_f);
    h->kernel = h->eo_ok ? BK_KERNEL_SWEEP : BK_KERNEL_COLUMN;
    if (!h->eo_ok && !column_fits(*h)) {
        delete h;
        return BK_ERR_ARG;
    }
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    int rc = BK_OK;
    const size_t nb = size_t(h->n);
    rc |= ck(cudaMalloc(&h->tiles, sizeof(MultiTile) * (h->ntiles > 0 ? h->ntiles : 1)));
    rc |= ck(cudaMalloc(&h->r64, 8 * (nb + 1)));
    rc |= ck(cudaMalloc(&h->r32, 4 * (nb + 4)));
    rc |= ck(cudaMalloc(&h->p32, 4 * (nb + 4)));
    rc |= ck(cudaMalloc(&h->Ap32, 4 * (nb + 4)));
    rc |= ck(cudaMalloc(&h->d32, 4 * (nb + 4)));
    rc |= ck(cudaMalloc(&h->invd, 4 * (nb + 4)));
    rc |= ck(cudaMalloc(&h->part, 8 * (kRedBlocks > kMaxDotParts ? kRedBlocks : kMaxDotParts)));
    rc |= ck(cudaMalloc(&h->sc, 8 * S_NSCAL));
    rc |= ck(cudaMalloc(&h->beta, 8 * 2));
    if (rc == BK_OK && h->ntiles > 0)
        rc = ck(cudaMemcpyAsync(h->tiles, h->htiles.data(), sizeof(MultiTile) * h->ntiles, cudaMemcpyHostToDevice, s));
    if (rc == BK_OK) rc = ck(cudaStreamSynchronize(s));
    if (rc != BK_OK) {
        bk_hplan_destroy(h);
        return BK_ERR_CUDA;
    }
    *out = h;
    return BK_OK;
}

int bk_hplan_destroy(bk_hplan_t h)
{
    if (!h) return BK_OK;
    free_graph(h);
    cudaFree(h->tiles);
    cudaFree(h->tiles64);
    cudaFree(h->r64);
    cudaFree(h->r32);
    cudaFree(h->p32);
    cudaFree(h->Ap32);
    cudaFree(h->d32);
    cudaFree(h->invd);
    cudaFree(h->part);
    cudaFree(h->sc);
    cudaFree(h->beta);
    delete h;
    return BK_OK;
}

long long bk_hplan_size(bk_hplan_t h, int what)
{
    if (!h) return -1;
    if (what == 0) return h->n;
    if (what == 1) return h->ng;
    if (what == 2) return h->ntiles;
    if (what == 3) return h->kernel;
    if (what == 4) {
        int ub = 0, gb = 0, wb = 0;
        return MultiFF::smem(h->e_ff, ub, gb, wb);
    }
    if (what == 5) return smem_f32<EngMixed>(h->e_f32);
    if (what == 6) return h->e_f32.block;
    if (what == 7) return h->e_f32.gstage;
    if (what == 8) return h->tiles64 ? h->ntiles64 : h->ntiles;
    if (what == 9) return h->e_ff.block;
    return -1;
}

int bk_hplan_set_fp64_shape(bk_hplan_t h, const int* elems_per_tile, int threads, bk_stream_t stream)
{
    if (!h) return BK_ERR_NULL;
    if (threads != 0 && (threads < 64 || threads > kNT || threads % 32 != 0)) return BK_ERR_ARG;
    MultiSeg seg[kMultiNQ];
    for (int s = 0; s < h->nseg; ++s) {
        seg[s] = h->seg[s];
        if (elems_per_tile && elems_per_tile[s] != 0) {
            const int q = seg[s].q;
            if (elems_per_tile[s] < 0 || elems_per_tile[s] * q * q > kMaxTileLines) return BK_ERR_ARG;
            seg[s].eb = elems_per_tile[s];
        }
    }
    MultiTile* dev = nullptr;
    int ntiles = 0;
    if (elems_per_tile) {
        const std::vector<MultiTile> t = make_tiles(seg, h->nseg);
        ntiles = int(t.size());
        cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
        if (ck(cudaMalloc(&dev, sizeof(MultiTile) * (ntiles > 0 ? ntiles : 1)))) return BK_ERR_CUDA;
        int rc = BK_OK;
        if (ntiles > 0)
            rc = ck(cudaMemcpyAsync(dev, t.data(), sizeof(MultiTile) * ntiles, cudaMemcpyHostToDevice, s));
        if (rc == BK_OK) rc = ck(cudaStreamSynchronize(s));
        if (rc != BK_OK) {
            cudaFree(dev);
            return rc;
        }
    }
    // the old list may still be read by FP64 applies queued on any stream
    if (h->tiles64) {
        if (ck(cudaDeviceSynchronize())) {
            cudaFree(dev);
            return BK_ERR_CUDA;
        }
        cudaFree(h->tiles64);
    }
    h->tiles64 = dev;
    h->ntiles64 = ntiles;
    for (int s = 0; s < h->nseg; ++s) h->e_dfma.seg[s].eb = h->e_ff.seg[s].eb = seg[s].eb;
    h->e_dfma.block = h->e_ff.block = elems_per_tile ? threads : h->e_f32.block;
    return BK_OK;
}

int bk_hplan_set_shape(bk_hplan_t h, int threads, int gstage)
{
    if (!h) return BK_ERR_NULL;
    if (threads != 0 && (threads < 64 || threads > kNT || threads % 32 != 0)) return BK_ERR_ARG;
    if (gstage != 0 && gstage != 1) return BK_ERR_ARG;
    if (threads != h->e_f32.block || gstage != h->e_f32.gstage) {
        free_graph(h);
        h->e_dfma.block = h->e_ff.block = h->e_f32.block = threads;
        h->e_dfma.gstage = h->e_ff.gstage = h->e_f32.gstage = gstage;
    }
    return BK_OK;
}

int bk_hplan_set_kernel(bk_hplan_t h, int kernel)
{
    if (!h) return BK_ERR_NULL;
    int k;
    if (kernel == BK_KERNEL_AUTO) k = h->eo_ok ? BK_KERNEL_SWEEP : BK_KERNEL_COLUMN;
    else if (kernel == BK_KERNEL_COLUMN) k = BK_KERNEL_COLUMN;
    else if (kernel == BK_KERNEL_SWEEP && h->eo_ok) k = BK_KERNEL_SWEEP;
    else return BK_ERR_ARG;
    if (k == BK_KERNEL_COLUMN && !column_fits(*h)) return BK_ERR_ARG;
    if (k != h->kernel) {
        free_graph(h);
        h->kernel = k;
    }
    return BK_OK;
}

int bk_hplan_apply(bk_hplan_t h, const void* G, const void* mass, double lambda, const void* u, void* v, int prec,
                   int engine, bk_stream_t stream)
{
    if (!h) return BK_ERR_NULL;
    if (h->n == 0) return BK_OK;
    if (!G || !u || !v) return BK_ERR_NULL;
    if ((reinterpret_cast<uintptr_t>(G) | reinterpret_cast<uintptr_t>(u) | reinterpret_cast<uintptr_t>(v) |
         reinterpret_cast<uintptr_t>(mass)) & 15)
        return BK_ERR_ALIGN;
    int eng;
    if (prec == BK_PREC_FP32) eng = 2;
    else if (prec == BK_PREC_MIXED) eng = 3;
    else if (prec == BK_PREC_FP64) eng = (engine == BK_ENGINE_DFMA) ? 0 : 1;
    else return BK_ERR_PREC;
    if (prec == BK_PREC_FP64 && engine != BK_ENGINE_AUTO && engine != BK_ENGINE_DFMA && engine != BK_ENGINE_FF)
        return BK_ERR_PREC;
    if (dev_ctx().status == nullptr) return BK_ERR_CUDA;
    return apply_plan(h, eng, G, mass, lambda, u, v, reinterpret_cast<cudaStream_t>(stream));
}

int bk_hplan_diagonal(bk_hplan_t h, const void* G, const void* mass, double lambda, double* diag, bk_stream_t stream)
{
    if (!h) return BK_ERR_NULL;
    if (h->n == 0) return BK_OK;
    if (!G || !diag) return BK_ERR_NULL;
    if ((reinterpret_cast<uintptr_t>(G) | reinterpret_cast<uintptr_t>(mass) | reinterpret_cast<uintptr_t>(diag)) & 15)
        return BK_ERR_ALIGN;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    for (int sg = 0; sg < h->nseg; ++sg) {
        const long long np = h->seg[sg].E * h->seg[sg].q * h->seg[sg].q * h->seg[sg].q;
        if (np == 0) continue;
        diag_kernel<double, double, false><<<grid_n(np), 256, 0, s>>>(h->p_dfma, sg, static_cast<const double*>(G),
                                                                      static_cast<const double*>(mass), lambda, diag);
    }
    return ck(cudaGetLastError());
}

int bk_hplan_cg(bk_hplan_t h, const void* G64, const void* mass64, const void* G32, const void* mass32,
                double lambda, const double* f, double* x, const bk_cg_options* opt, bk_cg_stats* stats,
                bk_stream_t stream)
{
    if (!h || !f || !x || !G64 || !G32) return BK_ERR_NULL;
    bk_cg_options o;
    o.rtol = 1e-10;
    o.max_outer = 8;
    o.inner_rtol = 1e-5;
    o.max_inner = 10000;
    o.precond = BK_PRECOND_JACOBI;
    if (opt) o = *opt;
    if (!(o.rtol > 0) || !(o.inner_rtol > 0) || o.max_outer < 1 || o.max_inner < 1) return BK_ERR_ARG;
    if (o.precond != BK_PRECOND_NONE && o.precond != BK_PRECOND_JACOBI) return BK_ERR_ARG;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    const long long n = h->n;
    int rc;
    if (dev_ctx().status == nullptr) return BK_ERR_CUDA;
    if (!h->inner_exec || h->g_key[0] != G32 || h->g_key[1] != mass32 || h->key_lambda != lambda ||
        h->key_precond != o.precond) {
        if ((rc = fill_precond(h, G32, mass32, lambda, o.precond, s))) return rc;
        if ((rc = build_inner_graph(h, G32, mass32, lambda, o.precond, s))) return rc;
    }
    const double sc_init[2] = {o.inner_rtol * o.inner_rtol, double(o.max_inner)};
    if ((rc = ck(cudaMemcpyAsync(h->sc + S_TOL2, sc_init, 2 * sizeof(double), cudaMemcpyHostToDevice, s)))) return rc;
    // |f|^2
    dot64_partial_kernel<<<kRedBlocks, kRedThreads, 0, s>>>(n, f, f, h->part);
    sum_to_kernel<<<1, kRedThreads, 0, s>>>(h->part, kRedBlocks, h->sc + S_FN2);
    double hs[S_NSCAL];
    int outer = 0, inner_total = 0;
    double relres = 0.0;
    for (;;) {
        // r = f - A x (FP64-accurate apply), |r|
        if ((rc = apply_plan(h, 1, G64, mass64, lambda, x, h->r64, s))) return rc;
        res64_kernel<<<kRedBlocks, kRedThreads, 0, s>>>(n, f, h->r64, h->part);
        norm_kernel<<<1, kRedThreads, 0, s>>>(h->part, kRedBlocks, h->sc);
        if ((rc = ck(cudaMemcpyAsync(hs, h->sc, sizeof(hs), cudaMemcpyDeviceToHost, s)))) return rc;
        if ((rc = ck(cudaStreamSynchronize(s)))) return rc;
        if (outer > 0) inner_total += int(hs[S_IT]);
        relres = hs[S_FN2] > 0 ? std::sqrt(hs[S_RN2] / hs[S_FN2]) : std::sqrt(hs[S_RN2]);
        if (relres <= o.rtol || outer >= o.max_outer || !(relres == relres)) break;
        // inner solve A d = r / |r| in FP32 (one graph launch), x += |r| d
        if ((rc = ck(cudaGraphLaunch(h->inner_exec, s)))) return rc;
        cg_correct_kernel<<<grid_n(n), 256, 0, s>>>(n, h->sc, h->d32, x);
        ++outer;
    }
    if (stats) {
        stats->outer = outer;
        stats->inner = inner_total;
        stats->relres = relres;
    }
    int st = 0;
    if ((rc = bk_device_status(&st, 0, stream))) return rc;
    if (st != BK_OK) return st;
    return relres <= o.rtol ? BK_OK : BK_ERR_NOCONV;
}

}  // extern "C"
