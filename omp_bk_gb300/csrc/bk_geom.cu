// bk_geom.cu -- seeded synthetic inputs of the benchmark configurations, built
// on the GPU in FP64: uniform and log-normal fields, and the geometric data of
// two meshes (qdata = w detJ, G = w detJ J^-1 J^-T, the collocated mass).  The
// reference has no geometry at all (its drivers use constant G = 2, JxW = 1,
// or the LCG of include/bk_common.h:92-107); these generators are written from
// the definitions:
//   affine mesh: element e maps [-1,1]^3 by x = c_e + (h/2)(I + delta_e) xi,
//     delta_e entries seeded U[-pert, pert] (detJ constant per element);
//   trilinear mesh: a uniform grid of spacing h whose vertices are jittered by
//     seeded U[-jit h, jit h] per coordinate, each element the trilinear map of
//     its 8 vertices (neighbouring elements share vertices: a conforming mesh).
// Random numbers: value i of stream `seed` is splitmix64(splitmix64(seed) + i)
// (Steele, Lea, Flood 2014), its top 53 bits as a uniform in [0, 1): the same
// on host and device, independent of launch shape.
#include <cmath>
#include <cstdint>

#include <cuda_runtime.h>

#include "bk_data.h"

namespace {

__host__ __device__ __forceinline__ uint64_t splitmix64(uint64_t z)
{
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

__host__ __device__ __forceinline__ double uniform01(uint64_t key, uint64_t i)
{
    return double(splitmix64(key + i) >> 11) * (1.0 / 9007199254740992.0);
}

constexpr int kMaxPts = 10;

struct Rule {
    double x[kMaxPts];
    double w[kMaxPts];
};

template <class T>
__global__ void fill_uniform_kernel(T* out, long long n, uint64_t key, double lo, double hi)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        out[i] = T(lo + (hi - lo) * uniform01(key, uint64_t(i)));
    }
}

// exp(sigma * z), z standard normal by Box-Muller from two uniforms
template <class T>
__global__ void fill_lognormal_kernel(T* out, long long n, uint64_t key, double sigma)
{
    const double two_pi = 6.283185307179586;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const double u1 = 1.0 - uniform01(key, 2 * uint64_t(i));   // (0, 1]
        const double u2 = uniform01(key, 2 * uint64_t(i) + 1);
        const double z = sqrt(-2.0 * log(u1)) * cos(two_pi * u2);
        out[i] = T(exp(sigma * z));
    }
}

__device__ __forceinline__ void metric(const double J[3][3], double w, double g[6], double& detJ)
{
    // J[a][b] = d x_a / d xi_b
    const double c00 = J[1][1] * J[2][2] - J[1][2] * J[2][1];
    const double c01 = J[1][2] * J[2][0] - J[1][0] * J[2][2];
    const double c02 = J[1][0] * J[2][1] - J[1][1] * J[2][0];
    detJ = J[0][0] * c00 + J[0][1] * c01 + J[0][2] * c02;
    const double id = 1.0 / detJ;
    // inverse K = J^-1, K[b][a] = d xi_b / d x_a
    double K[3][3];
    K[0][0] = c00 * id;
    K[1][0] = c01 * id;
    K[2][0] = c02 * id;
    K[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) * id;
    K[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) * id;
    K[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) * id;
    K[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) * id;
    K[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) * id;
    K[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) * id;
    const double s = w * detJ;
    const int ia[6] = {0, 0, 0, 1, 1, 2};
    const int ib[6] = {0, 1, 2, 1, 2, 2};
    for (int f = 0; f < 6; ++f) {
        const int a = ia[f], b = ib[f];
        g[f] = s * (K[a][0] * K[b][0] + K[a][1] * K[b][1] + K[a][2] * K[b][2]);
    }
}

__device__ __forceinline__ long long g_offset(int Q, int layout, int i, int j, int f, int k)
{
    if (layout == 0) return ((f * Q + i) * Q + j) * Q + k;
    if (layout == 1) return ((i * Q + j) * 6 + f) * Q + k;
    return ((f * Q + k) * Q + i) * Q + j;
}

// One thread per (element, point).
__global__ void geom_affine_kernel(int Q, long long E, const Rule rule, uint64_t key, double h, double pert,
                                   double* qdata, double* G, int layout)
{
    const long long Q3 = (long long)Q * Q * Q;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < E * Q3;
         t += (long long)gridDim.x * blockDim.x) {
        const long long e = t / Q3;
        const int x = int(t - e * Q3);
        const int i = x / (Q * Q), j = (x / Q) % Q, k = x % Q;
        double J[3][3];
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b)
                J[a][b] = 0.5 * h * ((a == b ? 1.0 : 0.0) + pert * (2.0 * uniform01(key, uint64_t(e) * 9 + a * 3 + b) - 1.0));
        const double w = rule.w[i] * rule.w[j] * rule.w[k];
        double g[6], detJ;
        metric(J, w, g, detJ);
        if (qdata) qdata[t] = w * detJ;
        if (G) {
            for (int f = 0; f < 6; ++f) G[e * 6 * Q3 + g_offset(Q, layout, i, j, f, k)] = g[f];
        }
    }
}

__device__ __forceinline__ double vertex_coord(uint64_t key, double h, double jit, long long vx, long long vy,
                                               long long vz, int nx, int ny, int c)
{
    const long long vid = vx + (nx + 1LL) * (vy + (ny + 1LL) * vz);
    const long long base = (c == 0) ? vx : (c == 1 ? vy : vz);
    return h * (double(base) + jit * (2.0 * uniform01(key, uint64_t(vid) * 3 + c) - 1.0));
}

__global__ void geom_trilinear_kernel(int Q, long long E, int nx, int ny, const Rule rule, uint64_t key, double h,
                                      double jit, double* G, int layout, double* mass, double* coords)
{
    const long long Q3 = (long long)Q * Q * Q;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < E * Q3;
         t += (long long)gridDim.x * blockDim.x) {
        const long long e = t / Q3;
        const int x = int(t - e * Q3);
        const int i = x / (Q * Q), j = (x / Q) % Q, k = x % Q;
        const long long ex = e % nx, ey = (e / nx) % ny, ez = e / ((long long)nx * ny);
        const double xi[3] = {rule.x[i], rule.x[j], rule.x[k]};
        double J[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
        double X[3] = {0, 0, 0};
        for (int v = 0; v < 8; ++v) {
            const int a = v & 1, b = (v >> 1) & 1, c = (v >> 2) & 1;
            // shape function prod (1 +- xi)/2 and its gradient
            const double s0 = a ? 0.5 * (1 + xi[0]) : 0.5 * (1 - xi[0]);
            const double s1 = b ? 0.5 * (1 + xi[1]) : 0.5 * (1 - xi[1]);
            const double s2 = c ? 0.5 * (1 + xi[2]) : 0.5 * (1 - xi[2]);
            const double d0 = a ? 0.5 : -0.5, d1 = b ? 0.5 : -0.5, d2 = c ? 0.5 : -0.5;
            const double dN[3] = {d0 * s1 * s2, s0 * d1 * s2, s0 * s1 * d2};
            for (int cc = 0; cc < 3; ++cc) {
                const double Xv = vertex_coord(key, h, jit, ex + a, ey + b, ez + c, nx, ny, cc);
                X[cc] += s0 * s1 * s2 * Xv;
                for (int d = 0; d < 3; ++d) J[cc][d] += Xv * dN[d];
            }
        }
        const double w = rule.w[i] * rule.w[j] * rule.w[k];
        double g[6], detJ;
        metric(J, w, g, detJ);
        if (G) {
            for (int f = 0; f < 6; ++f) G[e * 6 * Q3 + g_offset(Q, layout, i, j, f, k)] = g[f];
        }
        if (mass) mass[t] = w * detJ;
        if (coords) {
            coords[3 * t + 0] = X[0];
            coords[3 * t + 1] = X[1];
            coords[3 * t + 2] = X[2];
        }
    }
}

// Physical coordinates of the affine mesh at the points of `rule`: element e
// of an nx x ny x .. grid of spacing h is centred at ((ex, ey, ez) + 1/2) h.
__global__ void coords_affine_kernel(int Q, long long E, int nx, int ny, const Rule rule, uint64_t key, double h,
                                     double pert, double* coords)
{
    const long long Q3 = (long long)Q * Q * Q;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < E * Q3;
         t += (long long)gridDim.x * blockDim.x) {
        const long long e = t / Q3;
        const int x = int(t - e * Q3);
        const int i = x / (Q * Q), j = (x / Q) % Q, k = x % Q;
        const long long ex = e % nx, ey = (e / nx) % ny, ez = e / ((long long)nx * ny);
        const double c[3] = {(ex + 0.5) * h, (ey + 0.5) * h, (ez + 0.5) * h};
        const double xi[3] = {rule.x[i], rule.x[j], rule.x[k]};
        for (int a = 0; a < 3; ++a) {
            double s = c[a];
            for (int b = 0; b < 3; ++b) {
                const double Jab =
                    0.5 * h * ((a == b ? 1.0 : 0.0) + pert * (2.0 * uniform01(key, uint64_t(e) * 9 + a * 3 + b) - 1.0));
                s += Jab * xi[b];
            }
            coords[3 * t + a] = s;
        }
    }
}

template <class A, class B>
__global__ void convert_kernel(const A* in, B* out, long long n)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        out[i] = B(in[i]);
}

int grid1d(long long n)
{
    const long long g = (n + 255) / 256;
    return int(g < 152LL * 64 ? (g > 0 ? g : 1) : 152LL * 64);
}

bool load_rule(int Q, const double* x, const double* w, Rule& r)
{
    if (Q < 1 || Q > kMaxPts || !x || !w) return false;
    for (int i = 0; i < Q; ++i) {
        r.x[i] = x[i];
        r.w[i] = w[i];
    }
    return true;
}

int launched() { return cudaGetLastError() == cudaSuccess ? BK_OK : BK_ERR_CUDA; }

}  // namespace

extern "C" {

// out[i] = lo + (hi - lo) U_i, U_i the i-th uniform of stream `seed`;
// f64 != 0: out is double, else float.
int bk_fill_uniform(void* out, long long n, unsigned long long seed, double lo, double hi, int f64,
                    bk_stream_t stream)
{
    if (n < 0) return BK_ERR_SIZE;
    if (n == 0) return BK_OK;
    if (!out) return BK_ERR_NULL;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    const uint64_t key = splitmix64(seed);
    if (f64)
        fill_uniform_kernel<double><<<grid1d(n), 256, 0, s>>>(static_cast<double*>(out), n, key, lo, hi);
    else
        fill_uniform_kernel<float><<<grid1d(n), 256, 0, s>>>(static_cast<float*>(out), n, key, lo, hi);
    return launched();
}

// out[i] = exp(sigma z_i), z_i standard normal (log-normal coefficient).
int bk_fill_lognormal(void* out, long long n, unsigned long long seed, double sigma, int f64, bk_stream_t stream)
{
    if (n < 0) return BK_ERR_SIZE;
    if (n == 0) return BK_OK;
    if (!out) return BK_ERR_NULL;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    const uint64_t key = splitmix64(seed);
    if (f64)
        fill_lognormal_kernel<double><<<grid1d(n), 256, 0, s>>>(static_cast<double*>(out), n, key, sigma);
    else
        fill_lognormal_kernel<float><<<grid1d(n), 256, 0, s>>>(static_cast<float*>(out), n, key, sigma);
    return launched();
}

// Affine mesh: qdata (E x Q^3, may be NULL) and G (E x 6 x Q^3 in `layout`,
// may be NULL) at the points x / weights w (host, Q values).
int bk_geom_affine(int Q, long long E, const double* x, const double* w, unsigned long long seed, double h,
                   double pert, double* qdata, double* G, int layout, bk_stream_t stream)
{
    Rule r;
    if (!load_rule(Q, x, w, r) || layout < 0 || layout > 2) return BK_ERR_ARG;
    if (E < 0) return BK_ERR_SIZE;
    if (E == 0) return BK_OK;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    geom_affine_kernel<<<grid1d(E * Q * Q * Q), 256, 0, s>>>(Q, E, r, splitmix64(seed), h, pert, qdata, G, layout);
    return launched();
}

// Physical coordinates (E x Q^3 x 3) of the affine mesh (nx x ny x .. grid).
int bk_coords_affine(int Q, long long E, int nx, int ny, const double* x, unsigned long long seed, double h,
                     double pert, double* coords, bk_stream_t stream)
{
    Rule r;
    if (!load_rule(Q, x, x, r) || nx < 1 || ny < 1 || !coords) return BK_ERR_ARG;
    if (E < 0) return BK_ERR_SIZE;
    if (E == 0) return BK_OK;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    coords_affine_kernel<<<grid1d(E * Q * Q * Q), 256, 0, s>>>(Q, E, nx, ny, r, splitmix64(seed), h, pert, coords);
    return launched();
}

// Jittered trilinear mesh on an nx x ny x .. grid: G (layout), the collocated
// mass w detJ and the physical coordinates (each may be NULL).
int bk_geom_trilinear(int Q, long long E, int nx, int ny, const double* x, const double* w, unsigned long long seed,
                      double h, double jit, double* G, int layout, double* mass, double* coords, bk_stream_t stream)
{
    Rule r;
    if (!load_rule(Q, x, w, r) || layout < 0 || layout > 2 || nx < 1 || ny < 1) return BK_ERR_ARG;
    if (E < 0) return BK_ERR_SIZE;
    if (E == 0) return BK_OK;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    geom_trilinear_kernel<<<grid1d(E * Q * Q * Q), 256, 0, s>>>(Q, E, nx, ny, r, splitmix64(seed), h, jit, G, layout,
                                                                 mass, coords);
    return launched();
}

// double -> float (to_f32 != 0) or float -> double.
int bk_convert(const void* in, void* out, long long n, int to_f32, bk_stream_t stream)
{
    if (n < 0) return BK_ERR_SIZE;
    if (n == 0) return BK_OK;
    if (!in || !out) return BK_ERR_NULL;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    if (to_f32)
        convert_kernel<double, float><<<grid1d(n), 256, 0, s>>>(static_cast<const double*>(in), static_cast<float*>(out), n);
    else
        convert_kernel<float, double><<<grid1d(n), 256, 0, s>>>(static_cast<const float*>(in), static_cast<double*>(out), n);
    return launched();
}

}  // extern "C"
