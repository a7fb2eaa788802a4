// bk_kernels.cuh -- the BK1 / BK3 / BK5 operator kernels for sm_103a.
//
// One thread block processes a batch of EB elements at a time (grid-stride
// over the batches).  Per batch:
//   1. stage: the batch's slices of u and of the geometric data (qdata or G)
//      are contiguous in HBM (element-major E-vectors); each is copied into
//      shared memory by one 1-D TMA bulk copy (cp.async.bulk, completion on an
//      mbarrier with a bounded wait), rounded out to 16-byte boundaries inside
//      the array, so any element count and any odd extent is staged without
//      synchronous loads (stage_issue).
//   2. load pass: u is converted to the working type (float-float split for
//      the FP64 engine) into a padded work box -- or, for BK1/BK3 forms that
//      need no conversion, read by the first interpolation straight from the
//      stage.
//   3. sweeps: every 1-D contraction (interpolation with B, derivative with
//      D, and their transposes) is a "sweep" of one direction: one thread per
//      line of the box loads the line into registers, forms all outputs of the
//      line and writes them back.  Steps along k, whose lines one thread owns,
//      are chained in registers (kline_pass).  The 1-D matrices are kernel
//      parameters (__grid_constant__), so every coefficient is an operand of
//      the FMA straight from the constant bank.
//   4. pointwise: qdata (BK1) or G (BK3, BK5, with the optional coefficient k
//      of BK3) at every quadrature point.
//   5. the result is written to HBM with coalesced stores (from the box, or
//      from the last interpolation's registers).
// Work boxes are padded (row stride ZP, plane stride PS, element stride) per
// Q from a model of the warps' shared-memory wavefronts (bk5_box, bk3_box);
// BK3's FP32-storage box at Q = 8 also swizzles its rows and moves k lines
// as 128-bit accesses (WBox3, BoxLine, line_load / line_store).
#pragma once

#include <cstdint>
#include <type_traits>

#include "bk_device.cuh"
#include "bk_engine.cuh"

namespace bkg {

constexpr int kMaxQ = 10;

// ---- padded work boxes ---------------------------------------------------------

// The first strides of a Q x Q x Q work box of `vbytes`-byte values (now
// the fallback outside the tables below and the baseline the tables are
// scored against): rows of odd length keep the contiguous lines of
// direction 2 on distinct banks; the plane stride is chosen so that the
// lines of direction 1 split evenly across the banks; elements Q planes
// apart.
constexpr int box_zp(int q) { return (q % 2 == 0) ? q + 1 : q; }
constexpr int box_ps(int q, int vbytes)
{
    // plane stride in words of the value: for 8-byte values aim at PS = 8
    // (mod 16), for 4-byte values at PS = 8 (mod 32) or 16 (mod 32)
    return (vbytes == 8) ? ((q * box_zp(q)) % 16 == 8 ? q * box_zp(q) : q * box_zp(q) + ((24 - (q * box_zp(q)) % 16) % 16))
                         : ((q * box_zp(q)) % 32 == 8 ? q * box_zp(q) : q * box_zp(q) + ((40 - (q * box_zp(q)) % 32) % 32));
}

// The BK5 work box (the sweep kernel and the mixed-order Helmholtz kernel):
// row stride, plane stride and element stride (values) per Q and value size,
// each the minimum of a model of the warps' shared-memory wavefronts over
// the box's access patterns, averaged over the elements per block that occur
// (omp_bk_gb300/box_model.py).  For small Q a warp spans several elements,
// so the element stride matters as much as the row and plane strides.
// 4-byte values (FP32 storage, no direction groups: the load and last
// passes by i lines, the pointwise stage by k lines, the thread-per-line
// sweeps of the three directions; --op 52) and 8-byte values (the dense
// walks of the direction-parallel blocks and the pointwise walk in G's
// (k, i, j) order; --op 5).  Model wavefronts per access (1 =
// conflict-free) against the first strides (box_zp, box_ps):
//   4-byte values, Q = 2..9: 1.10 1.39 1.20 1.38 1.34 1.36 1.36 1.13
//                   (first:  3.00 2.53 2.00 1.88 1.75 1.62 1.36 1.75)
//   8-byte values, Q = 2..9: 1.36 1.62 1.18 1.41 1.44 1.43 1.36 1.23
//                   (first:  3.09 2.55 2.00 1.80 1.96 1.65 1.36 1.62)
constexpr int bk5_box(int q, int vbytes, int what)   // what: 0 ZP, 1 PS, 2 element stride
{
    // {ZP, PS, element stride} for q = 2..9
    constexpr int t4[8][3] = {{2, 15, 36}, {3, 9, 27}, {4, 19, 80}, {5, 25, 125},
                              {7, 42, 252}, {7, 49, 343}, {9, 72, 576}, {9, 81, 729}};
    constexpr int t8[8][3] = {{4, 8, 18}, {3, 9, 27}, {4, 19, 76}, {5, 25, 125},
                              {9, 54, 324}, {7, 49, 343}, {9, 72, 576}, {9, 81, 737}};
    return (q < 2 || q > 9) ? (what == 0 ? box_zp(q) : (what == 1 ? box_ps(q, vbytes) : q * box_ps(q, vbytes)))
                            : (vbytes == 8 ? t8[q - 2][what] : t4[q - 2][what]);
}

// The work box of BK1, BK3 and the BK3 adjoint (P = Q - 1 nodes, Q points):
// the same model over their walks (the dense P^3 load and store, the
// interpolation sweeps through the (Q,P,P) and (Q,Q,P) boxes and back, the
// gradient sweeps and the dense pointwise walk; box_model.py --op 3).  At
// 4-byte Q = 8 the model of the flow fused along k (--op 31) picks
// {8, 71, 568}: BK3 p=6 mixed 110.2 against 109.8 GDoF/s with the first
// strides (before the fusion the same box had measured 83.0 against 87.6);
// BK3's FP32-storage forms now use the swizzled box below at Q = 8, the
// table's entry serves BK1 and the adjoint.  Model wavefronts per access,
// Q = 3..10, against the first strides:
//   4-byte values: 1.45 1.55 1.48 1.67 1.64 1.49 1.31 1.48
//                 (2.49 2.21 1.96 1.86 1.73 1.49 1.61 1.81)
//   8-byte values: 1.44 1.25 1.43 1.58 1.58 1.55 1.40 1.47
//                 (2.51 2.08 1.81 1.90 1.69 1.55 1.58 1.90)
constexpr int bk3_box(int q, int vbytes, int what)   // what: 0 ZP, 1 PS, 2 element stride
{
    // {ZP, PS, element stride} for q = 3..10
    constexpr int b4[8][3] = {{3, 9, 27}, {4, 19, 80}, {5, 25, 125}, {6, 36, 216},
                              {7, 49, 343}, {8, 71, 568}, {9, 81, 729}, {10, 105, 1050}};
    constexpr int b8[8][3] = {{3, 9, 27}, {4, 19, 76}, {5, 25, 125}, {9, 54, 324},
                              {7, 54, 385}, {9, 72, 576}, {9, 81, 729}, {10, 105, 1050}};
    return (q < 3 || q > 10) ? (what == 0 ? box_zp(q) : (what == 1 ? box_ps(q, vbytes) : q * box_ps(q, vbytes)))
                             : (vbytes == 8 ? b8[q - 3][what] : b4[q - 3][what]);
}

// Row swizzle of a work box: value k of row (i, j) sits at i*PS + j*ZP +
// (k ^ swz(j)), swz(j) = X when bit SB of j is set, else 0 (X = 0: no
// swizzle).  With rows of 8 four-byte values (ZP = 8) a warp of 32 k lines
// (j = 0..7 at each of 4 i) otherwise meets rows j and j + 4 in the same
// banks; swapping the two halves of every row whose j has bit 2 set makes
// the 128-bit k-line accesses (VEC) and, with PS = 8 mod 32, the j-direction
// sweeps conflict-free.  Only BK3's FP32-storage forms at Q = 8 use it
// (box_model.py --op 32): the model's wavefronts per element fall from 612
// to 474, its shared-memory instructions from 424 to 344, and BK3 p=6 mixed
// went from 110.2 to 120.1 GDoF/s (same results).
constexpr int bk3_swz(int q, int vbytes) { return (q == 8 && vbytes == 4) ? 4 : 0; }

template <int Q, class V, bool SWZ = false>
struct WBox3 {
    static constexpr int X = SWZ ? bk3_swz(Q, int(sizeof(V))) : 0;
    static constexpr int SB = 2;
    static constexpr int ZP = X ? 8 : bk3_box(Q, int(sizeof(V)), 0);
    static constexpr int PS = X ? 72 : bk3_box(Q, int(sizeof(V)), 1);
    static constexpr int size = X ? 576 : bk3_box(Q, int(sizeof(V)), 2);
    // k lines as 128-bit accesses (16-byte aligned rows of 4-byte values)
    static constexpr bool VEC = X != 0;
    static_assert((Q - 1) * ZP + Q <= PS && (Q - 1) * PS + PS <= size, "box strides overlap");
    static_assert(!X || (Q <= 2 * X && ZP % 4 == 0 && PS % 4 == 0 && size % 4 == 0 && sizeof(V) == 4),
                  "swizzled rows hold two 16-byte halves");
    __device__ static __forceinline__ int swz(int j) { return X ? ((j >> SB) & 1) * X : 0; }
    __device__ static __forceinline__ int at(int i, int j, int k) { return i * PS + j * ZP + (k ^ swz(j)); }
};

template <int Q, class V>
struct WBox5 {
    static constexpr int X = 0, SB = 0;
    static constexpr bool VEC = false;
    static constexpr int ZP = bk5_box(Q, int(sizeof(V)), 0);
    static constexpr int PS = bk5_box(Q, int(sizeof(V)), 1);
    static constexpr int size = bk5_box(Q, int(sizeof(V)), 2);
    static_assert((Q - 1) * ZP + Q <= PS && (Q - 1) * PS + PS <= size, "box strides overlap");
    __device__ static __forceinline__ int swz(int) { return 0; }
    __device__ static __forceinline__ int at(int i, int j, int k) { return i * PS + j * ZP + k; }
};

// Addresses along one line of direction DIR of element e's box, the line
// given by its two other indices (a, b) in (i, j, k) order: (*this)(n) is
// the n-th value.  With a swizzle the index n, a compile-time constant in
// the unrolled loops, picks one of two per-line bases, so the swizzle costs
// no instruction per access:
//   DIR 0: (n, a, b) at b0 + n*PS (the row a is fixed);
//   DIR 1: (a, n, b) at b0 or b1 (b ^ X) + n*ZP, by bit SB of n;
//   DIR 2: (a, b, n) at b0 (= base + m) or b1 (= base - m) + n, by bit X of
//          n, m = swz(b): n ^ m = n + m or n - m.
template <class WB, int DIR>
struct BoxLine {
    int b0, b1;
    __device__ __forceinline__ BoxLine(int e, int a, int b)
    {
        const int eb = e * WB::size;
        if constexpr (DIR == 0) {
            b0 = eb + a * WB::ZP + (b ^ WB::swz(a));
            b1 = b0;
        } else if constexpr (DIR == 1) {
            b0 = eb + a * WB::PS + b;
            b1 = eb + a * WB::PS + (b ^ WB::X);
        } else {
            const int m = WB::swz(b);
            b0 = eb + a * WB::PS + b * WB::ZP + m;
            b1 = eb + a * WB::PS + b * WB::ZP - m;
        }
    }
    __device__ __forceinline__ int operator()(int n) const
    {
        if constexpr (DIR == 0) return b0 + n * WB::PS;
        else if constexpr (DIR == 1) return ((WB::X && ((n >> WB::SB) & 1)) ? b1 : b0) + n * WB::ZP;
        else return ((WB::X && (n & WB::X)) ? b1 : b0) + n;
    }
};

// The N values of a k line into registers / from registers; 128-bit
// accesses when the box allows them (WB::VEC: the line's halves are 16-byte
// aligned; the last half of a line of N < 8 values reads, or writes, the
// row's padding).
template <class WB, int N, class V>
__device__ __forceinline__ void line_load(const V* W, const BoxLine<WB, 2>& la, V (&x)[N])
{
    if constexpr (WB::VEC) {
        static_assert(sizeof(V) == 4 && N <= 8, "128-bit k lines of 4-byte values");
#pragma unroll
        for (int c = 0; c < (N + 3) / 4; ++c) {
            const float4 t = *reinterpret_cast<const float4*>(W + la(4 * c));
            const V tv[4] = {t.x, t.y, t.z, t.w};
#pragma unroll
            for (int q = 0; q < 4; ++q)
                if (4 * c + q < N) x[4 * c + q] = tv[q];
        }
    } else {
#pragma unroll
        for (int n = 0; n < N; ++n) x[n] = W[la(n)];
    }
}

template <class WB, int N, class V>
__device__ __forceinline__ void line_store(V* W, const BoxLine<WB, 2>& la, const V (&y)[N])
{
    if constexpr (WB::VEC) {
        static_assert(sizeof(V) == 4 && N <= 8, "128-bit k lines of 4-byte values");
#pragma unroll
        for (int c = 0; c < (N + 3) / 4; ++c) {
            V tv[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) tv[q] = y[(4 * c + q < N) ? 4 * c + q : N - 1];
            *reinterpret_cast<float4*>(W + la(4 * c)) = make_float4(tv[0], tv[1], tv[2], tv[3]);
        }
    } else {
#pragma unroll
        for (int n = 0; n < N; ++n) W[la(n)] = y[n];
    }
}

// ---- staging -------------------------------------------------------------------

// Shared-memory footprint (bytes) of a staged slice of n values of type S:
// 16 bytes of slack for the alignment of the slice's first value.
template <class S>
constexpr int stage_bytes(int n)
{
    return ((n * int(sizeof(S)) + 15) / 16) * 16 + 16;
}

// Issues the copy of src[0, n) (global) into the shared buffer `buf`
// (16-byte aligned, stage_bytes(n) long).  Returns where src[0] lands.
// `lim` is the end of the source array, whose start is 16-byte aligned: the
// TMA copy runs from src rounded down to 16 bytes (still inside the array)
// to the end rounded up to 16 bytes when that stays inside the array, so a
// slice that does not start or end on a 16-byte boundary still needs no
// synchronous loads; only a slice ending on the array's own unaligned end
// loads its last few values with plain loads.  Thread 0 issues the TMA
// part; every thread adds its bytes to *tx.
template <class S>
__device__ __forceinline__ S* stage_issue(void* buf, const S* src, int n, const S* lim, uint64_t* bar, uint32_t& tx,
                                          int tid, int nt);

// Where stage_issue(buf, src, ...) puts src[0]: the copy starts at src
// rounded down to 16 bytes, which lands on buf itself.
template <class S>
__device__ __forceinline__ const S* stage_at(const void* buf, const S* src)
{
    return reinterpret_cast<const S*>(static_cast<const char*>(buf) + (reinterpret_cast<uintptr_t>(src) & 15));
}

template <class S>
__device__ __forceinline__ S* stage_issue(void* buf, const S* src, int n, const S* lim, uint64_t* bar, uint32_t& tx,
                                          int tid, int nt)
{
    const uintptr_t a = reinterpret_cast<uintptr_t>(src);
    const uintptr_t b = a + uintptr_t(n) * sizeof(S);
    const uintptr_t a_dn = a & ~uintptr_t(15);
    const uintptr_t b_up = (b + 15) & ~uintptr_t(15);
    const uintptr_t b_cut = (b_up <= reinterpret_cast<uintptr_t>(lim)) ? b_up : (b & ~uintptr_t(15));
    // src[0] at offset (a mod 16), so that a_dn lands on buf itself
    S* dst = reinterpret_cast<S*>(static_cast<char*>(buf) + (a & 15));
    int plain0 = 0;   // first value loaded with plain loads
    if (b_cut > a_dn) {
        if (tid == 0) tma_load_1d(buf, reinterpret_cast<const void*>(a_dn), uint32_t(b_cut - a_dn), bar);
        tx += uint32_t(b_cut - a_dn);
        plain0 = b_cut >= b ? n : int((b_cut - a) / sizeof(S));
    }
    for (int i = plain0 + tid; i < n; i += nt) dst[i] = src[i];
    return dst;
}

// ---- sweeps --------------------------------------------------------------------

// Coefficient M(o, n) of a 1-D matrix stored row-major with leading dimension
// LD, optionally transposed.  `m` points into the kernel's parameter space.
template <class C, int LD, bool T>
struct Mat {
    const C* m;
    __device__ __forceinline__ C operator()(int o, int n) const { return T ? m[n * LD + o] : m[o * LD + n]; }
};

// Contract direction DIR of the box with extents (X, Y, Z) in `in` into `out`
// (extent NO along DIR): out(.., o, ..) = sum_n M(o, n) in(.., n, ..).  Boxes
// use the padded strides of WB whatever their extents; in == out is allowed
// (each line is read completely before it is written).  Lines of all `ne`
// elements are spread over the block's threads.
template <class Eng, class WB, int DIR, int X, int Y, int Z, int NO, class M>
__device__ __forceinline__ void sweep(const typename Eng::V* in, typename Eng::V* out, int ne, const M& mat,
                                      int tid, int nt)
{
    using V = typename Eng::V;
    using A = typename Eng::A;
    constexpr int NI = DIR == 0 ? X : (DIR == 1 ? Y : Z);
    constexpr int LB = DIR == 2 ? Y : Z;
    constexpr int L = (X * Y * Z) / NI;
    for (int w = tid; w < ne * L; w += nt) {
        const int e = w / L;
        const int l = w - e * L;
        const int a = l / LB;
        const int b = l - a * LB;
        const BoxLine<WB, DIR> la(e, a, b);
        V x[NI];
#pragma unroll
        for (int n = 0; n < NI; ++n) x[n] = in[la(n)];
#pragma unroll
        for (int o = 0; o < NO; ++o) {
            A acc = Eng::first(mat(o, 0), x[0]);
#pragma unroll
            for (int n = 1; n < NI; ++n) Eng::madd(acc, mat(o, n), x[n]);
            out[la(o)] = Eng::result(acc);
        }
    }
}

// Even-odd form of a square Q x Q matrix M with M(Q-1-o, Q-1-n) = -M(o, n)
// (the derivative matrix on points symmetric about 0, and its transpose):
// with H = Q/2, e(n) = x(n) + x(Q-1-n), d(n) = x(n) - x(Q-1-n) (n < H) and
// the middle value x(m) of an odd Q,
//   a(o) = sum_n A(o,n) e(n) + c(o) x(m),  b(o) = sum_n B(o,n) d(n),
//   out(o) = a(o) + b(o),  out(Q-1-o) = b(o) - a(o),  out(m) = sum_n r(n) d(n)
// with A = (M(o,n) + M(o,Q-1-n))/2, B = (M(o,n) - M(o,Q-1-n))/2, c(o) =
// M(o,m), r(n) = M(m,n): Q^2/2 multiply-adds instead of Q^2 (the classic
// even-odd decomposition of spectral-element codes).
template <class C, int Q>
struct EOMat {
    static constexpr int H = Q / 2;
    C A[H * H];
    C B[H * H];
    C c[H];
    C r[H];
};

// Host side: the even-odd form of M(o, n) = m[o*ld + n] (trans: m[n*ld + o]);
// true if M is centro-antisymmetric to within 1e-13 of its largest entry.
template <class C, int Q, class Conv>
inline bool make_eo(const double* m, bool trans, EOMat<C, Q>& out, Conv conv)
{
    constexpr int H = Q / 2;
    auto M = [&](int o, int n) { return trans ? m[n * Q + o] : m[o * Q + n]; };
    double big = 0, asym = 0;
    for (int o = 0; o < Q; ++o)
        for (int n = 0; n < Q; ++n) {
            big = big > (M(o, n) < 0 ? -M(o, n) : M(o, n)) ? big : (M(o, n) < 0 ? -M(o, n) : M(o, n));
            const double a = M(o, n) + M(Q - 1 - o, Q - 1 - n);
            asym = asym > (a < 0 ? -a : a) ? asym : (a < 0 ? -a : a);
        }
    for (int o = 0; o < H; ++o) {
        for (int n = 0; n < H; ++n) {
            out.A[o * H + n] = conv(0.5 * (M(o, n) + M(o, Q - 1 - n)));
            out.B[o * H + n] = conv(0.5 * (M(o, n) - M(o, Q - 1 - n)));
        }
        out.c[o] = conv((Q & 1) ? M(o, H) : 0.0);
        out.r[o] = conv((Q & 1) ? M(H, o) : 0.0);
    }
    return asym <= 1e-13 * big;
}

// Even-odd sweep of direction DIR of a Q x Q x Q box (in == out allowed);
// see EOMat.  When ADD is set, out(o) = M x + X(o) + Y(o) for the lines of
// direction 2 (BK5's last transposed derivative plus the other two terms).
// The Q outputs y of one line x through the square even-odd form m (see
// EOMat); x and y are register arrays of the caller.  LOOSE: the outputs
// as unevaluated pairs (Eng::sum_diff_loose), for outputs that are only
// summed or stored next, never multiplied.
template <class Eng, int Q, bool LOOSE = false, class EM>
__device__ __forceinline__ void eo_line(const typename Eng::V (&x)[Q], typename Eng::V (&y)[Q], const EM& m)
{
    using V = typename Eng::V;
    using A = typename Eng::A;
    constexpr int H = Q / 2;
    V ev[H > 0 ? H : 1], dv[H > 0 ? H : 1];
#pragma unroll
    for (int n = 0; n < H; ++n) {
        ev[n] = Eng::vadd_in(x[n], x[Q - 1 - n]);
        dv[n] = Eng::vsub_in(x[n], x[Q - 1 - n]);
    }
#pragma unroll
    for (int o = 0; o < H; ++o) {
        A aa = Eng::first(m.A[o * H], ev[0]), bb = Eng::first(m.B[o * H], dv[0]);
#pragma unroll
        for (int n = 1; n < H; ++n) {
            Eng::madd(aa, m.A[o * H + n], ev[n]);
            Eng::madd(bb, m.B[o * H + n], dv[n]);
        }
        if (Q & 1) Eng::madd(aa, m.c[o], x[H]);
        if constexpr (LOOSE)
            Eng::sum_diff_loose(aa, bb, y[o], y[Q - 1 - o]);   // a + b, b - a
        else
            Eng::sum_diff(aa, bb, y[o], y[Q - 1 - o]);
    }
    if constexpr ((Q & 1) != 0) {
        A t = Eng::first(m.r[0], dv[0]);
#pragma unroll
        for (int n = 1; n < H; ++n) Eng::madd(t, m.r[n], dv[n]);
        y[H] = LOOSE ? Eng::loose(t) : Eng::result(t);
    }
}

template <class Eng, class WB, int DIR, int Q, bool LOOSE = false, class EM>
__device__ __forceinline__ void sweep_eo(const typename Eng::V* in, typename Eng::V* out, int ne, const EM& m,
                                         int tid, int nt)
{
    using V = typename Eng::V;
    constexpr int LB = Q;
    constexpr int L = Q * Q;
    constexpr int SD = DIR == 0 ? WB::PS : (DIR == 1 ? WB::ZP : 1);
    static_assert(WB::X == 0, "unswizzled boxes");
    for (int w = tid; w < ne * L; w += nt) {
        const int e = w / L;
        const int l = w - e * L;
        const int a = l / LB;
        const int b = l - a * LB;
        int base = (DIR == 0) ? a * WB::ZP + b : (DIR == 1 ? a * WB::PS + b : a * WB::PS + b * WB::ZP);
        base += e * WB::size;
        V x[Q], y[Q];
#pragma unroll
        for (int n = 0; n < Q; ++n) x[n] = in[base + n * SD];
        eo_line<Eng, Q, LOOSE>(x, y, m);
#pragma unroll
        for (int o = 0; o < Q; ++o) out[base + o * SD] = y[o];
    }
}

// sweep_eo with the direction dir (0, 1, 2) given at run time: the line's
// strides are computed, not constants, so that one code body serves all
// three directions.  LOOSE: the outputs as unevaluated pairs (sum_diff_loose),
// for sweeps whose outputs are only summed next (the transposed derivatives).
template <class Eng, class WB, int Q, bool LOOSE = false, class EM>
__device__ __forceinline__ void sweep_eo_dyn(const typename Eng::V* in, typename Eng::V* out, int ne, const EM& m,
                                             int tid, int nt, int dir)
{
    using V = typename Eng::V;
    using A = typename Eng::A;
    constexpr int H = Q / 2;
    constexpr int L = Q * Q;
    static_assert(WB::X == 0, "unswizzled boxes");
    const int SD = dir == 0 ? WB::PS : (dir == 1 ? WB::ZP : 1);
    const int SA = dir == 0 ? WB::ZP : WB::PS;   // stride of the line's first index
    const int SB = dir == 2 ? WB::ZP : 1;        // stride of its second index
    for (int w = tid; w < ne * L; w += nt) {
        const int e = w / L;
        const int l = w - e * L;
        const int a = l / Q;
        const int b = l - a * Q;
        const V* pi = in + e * WB::size + a * SA + b * SB;
        V* po = out + e * WB::size + a * SA + b * SB;
        V x[Q];
#pragma unroll
        for (int n = 0; n < Q; ++n) x[n] = pi[n * SD];
        V ev[H > 0 ? H : 1], dv[H > 0 ? H : 1];
#pragma unroll
        for (int n = 0; n < H; ++n) {
            ev[n] = Eng::vadd_in(x[n], x[Q - 1 - n]);
            dv[n] = Eng::vsub_in(x[n], x[Q - 1 - n]);
        }
#pragma unroll
        for (int o = 0; o < H; ++o) {
            A aa = Eng::first(m.A[o * H], ev[0]), bb = Eng::first(m.B[o * H], dv[0]);
#pragma unroll
            for (int n = 1; n < H; ++n) {
                Eng::madd(aa, m.A[o * H + n], ev[n]);
                Eng::madd(bb, m.B[o * H + n], dv[n]);
            }
            if (Q & 1) Eng::madd(aa, m.c[o], x[H]);
            V s, d;
            if constexpr (LOOSE)
                Eng::sum_diff_loose(aa, bb, s, d);   // a + b, b - a
            else
                Eng::sum_diff(aa, bb, s, d);
            po[o * SD] = s;
            po[(Q - 1 - o) * SD] = d;
        }
        if (Q & 1) {
            A t = Eng::first(m.r[0], dv[0]);
#pragma unroll
            for (int n = 1; n < H; ++n) Eng::madd(t, m.r[n], dv[n]);
            po[H * SD] = Eng::result(t);
        }
    }
}

// Even-odd form of a rectangular NO x NI matrix with M(NO-1-o, NI-1-n) =
// SIGN M(o, n): the interpolation matrix between point sets symmetric about 0
// (SIGN = +1) and the derivative matrix (SIGN = -1), or their transposes.
// With HI = NI/2, HO = NO/2, e(n) = x(n) + x(NI-1-n), d(n) = x(n) - x(NI-1-n):
//   a(o) = sum_n A(o,n) e(n) + c(o) x(HI),   b(o) = sum_n B(o,n) d(n),
//   out(o) = a(o) + b(o),   out(NO-1-o) = SIGN (a(o) - b(o)),
// and for odd NO the middle row out(HO) = sum_n r(n) e(n) + rm x(HI) (SIGN
// +1) or sum_n r(n) d(n) (SIGN -1); x(HI) exists for odd NI only.
template <class C, int NO, int NI>
struct EORMat {
    static constexpr int HO = NO / 2;
    static constexpr int HI = NI / 2;
    C A[HO * HI > 0 ? HO * HI : 1];
    C B[HO * HI > 0 ? HO * HI : 1];
    C c[HO > 0 ? HO : 1];
    C r[HI > 0 ? HI : 1];
    C rm;
};

// Host side: the even-odd form of M(o, n) = m[o*ld + n] (trans: m[n*ld + o]);
// true if M(NO-1-o, NI-1-n) = sign M(o, n) to within 1e-13 of its largest
// entry.
template <class C, int NO, int NI, class Conv>
inline bool make_eor(const double* m, int ld, bool trans, int sign, EORMat<C, NO, NI>& out, Conv conv)
{
    constexpr int HO = NO / 2, HI = NI / 2;
    auto M = [&](int o, int n) { return trans ? m[n * ld + o] : m[o * ld + n]; };
    auto fab = [](double x) { return x < 0 ? -x : x; };
    double big = 0, dev = 0;
    for (int o = 0; o < NO; ++o)
        for (int n = 0; n < NI; ++n) {
            big = big > fab(M(o, n)) ? big : fab(M(o, n));
            const double a = M(NO - 1 - o, NI - 1 - n) - sign * M(o, n);
            dev = dev > fab(a) ? dev : fab(a);
        }
    for (int o = 0; o < HO; ++o) {
        for (int n = 0; n < HI; ++n) {
            out.A[o * HI + n] = conv(0.5 * (M(o, n) + M(o, NI - 1 - n)));
            out.B[o * HI + n] = conv(0.5 * (M(o, n) - M(o, NI - 1 - n)));
        }
        out.c[o] = conv((NI & 1) ? M(o, HI) : 0.0);
    }
    for (int n = 0; n < HI; ++n) out.r[n] = conv((NO & 1) ? M(HO, n) : 0.0);
    out.rm = conv(((NO & 1) && (NI & 1)) ? M(HO, HI) : 0.0);
    return dev <= 1e-13 * big;
}

// The NO outputs y of one line of NI inputs x through the even-odd form m
// (see EORMat); x and y are register arrays of the caller.  LOOSE as for
// eo_line.
template <class Eng, int NI, int NO, int SIGN, bool LOOSE = false, class EM>
__device__ __forceinline__ void eor_line(const typename Eng::V (&x)[NI], typename Eng::V (&y)[NO], const EM& m)
{
    using V = typename Eng::V;
    using A = typename Eng::A;
    constexpr int HI = NI / 2, HO = NO / 2;
    V ev[HI > 0 ? HI : 1], dv[HI > 0 ? HI : 1];
#pragma unroll
    for (int n = 0; n < HI; ++n) {
        ev[n] = Eng::vadd_in(x[n], x[NI - 1 - n]);
        dv[n] = Eng::vsub_in(x[n], x[NI - 1 - n]);
    }
    if constexpr ((NO & 1) != 0) {
        A t = Eng::first(m.r[0], SIGN > 0 ? ev[0] : dv[0]);
#pragma unroll
        for (int n = 1; n < HI; ++n) Eng::madd(t, m.r[n], SIGN > 0 ? ev[n] : dv[n]);
        if constexpr (SIGN > 0 && (NI & 1) != 0) Eng::madd(t, m.rm, x[HI]);
        y[HO] = LOOSE ? Eng::loose(t) : Eng::result(t);
    }
#pragma unroll
    for (int o = 0; o < HO; ++o) {
        A aa = Eng::first(m.A[o * HI], ev[0]), bb = Eng::first(m.B[o * HI], dv[0]);
#pragma unroll
        for (int n = 1; n < HI; ++n) {
            Eng::madd(aa, m.A[o * HI + n], ev[n]);
            Eng::madd(bb, m.B[o * HI + n], dv[n]);
        }
        if constexpr ((NI & 1) != 0) Eng::madd(aa, m.c[o], x[HI]);
        if constexpr (SIGN > 0 && LOOSE) {
            Eng::sum_diff_loose(bb, aa, y[o], y[NO - 1 - o]);   // b + a, a - b
        } else if constexpr (SIGN > 0) {
            Eng::sum_diff(bb, aa, y[o], y[NO - 1 - o]);
        } else if constexpr (LOOSE) {
            Eng::sum_diff_loose(aa, bb, y[o], y[NO - 1 - o]);   // a + b, b - a
        } else {
            Eng::sum_diff(aa, bb, y[o], y[NO - 1 - o]);
        }
    }
}

// Even-odd sweep of direction DIR of the (X, Y, Z) box into extent NO along
// DIR (see EORMat; in == out allowed).
template <class Eng, class WB, int DIR, int X, int Y, int Z, int NO, int SIGN, bool LOOSE = false, class EM>
__device__ __forceinline__ void sweep_eor(const typename Eng::V* in, typename Eng::V* out, int ne, const EM& m,
                                          int tid, int nt)
{
    using V = typename Eng::V;
    constexpr int NI = DIR == 0 ? X : (DIR == 1 ? Y : Z);
    constexpr int LB = DIR == 2 ? Y : Z;
    constexpr int L = (X * Y * Z) / NI;
    for (int w = tid; w < ne * L; w += nt) {
        const int e = w / L;
        const int l = w - e * L;
        const int a = l / LB;
        const int b = l - a * LB;
        const BoxLine<WB, DIR> la(e, a, b);
        V x[NI], y[NO];
        if constexpr (DIR == 2) {
            line_load<WB, NI>(in, la, x);
        } else {
#pragma unroll
            for (int n = 0; n < NI; ++n) x[n] = in[la(n)];
        }
        eor_line<Eng, NI, NO, SIGN, LOOSE>(x, y, m);
        if constexpr (DIR == 2) {
            line_store<WB, NO>(out, la, y);
        } else {
#pragma unroll
            for (int o = 0; o < NO; ++o) out[la(o)] = y[o];
        }
    }
}

// The first interpolation of BK1/BK3 straight from the dense staged u (P^3
// values of S per element, k fastest): lines along i, (j, k)
// consecutive across threads, so the stage reads are consecutive words; the
// Q outputs of each line go to the padded box `out` as (Q, P, P).  Replaces
// the load into a box and the sweep over it (one write and one read of
// every value less).
template <class Eng, class WB, int P, int Q, class EM>
__device__ __forceinline__ void interp0_from_dense(const typename Eng::S* us, typename Eng::V* out, int ne,
                                                   const EM& m, int tid, int nt)
{
    using V = typename Eng::V;
    constexpr int L = P * P;
    for (int w = tid; w < ne * L; w += nt) {
        const int e = w / L;
        const int l = w - e * L;
        const int j = l / P;
        const int kk = l - j * P;
        const typename Eng::S* src = us + e * (P * P * P) + j * P + kk;
        V x[P], y[Q];
#pragma unroll
        for (int n = 0; n < P; ++n) x[n] = Eng::load(src[n * P * P]);
        eor_line<Eng, P, Q, +1>(x, y, m);
        const BoxLine<WB, 0> la(e, j, kk);
#pragma unroll
        for (int o = 0; o < Q; ++o) out[la(o)] = y[o];
    }
}

// The last interpolation of BK1/BK3 (along i, (Q, P, P) box -> P^3) written
// straight to v in global memory: (j, k) consecutive across threads, so each
// output row is a coalesced store.  Replaces the sweep into a box and the
// store pass.
template <class Eng, class WB, int P, int Q, class EM>
__device__ __forceinline__ void interp0_to_dense(const typename Eng::V* in, typename Eng::S* __restrict__ v,
                                                 int ne, const EM& m, int tid, int nt)
{
    using V = typename Eng::V;
    constexpr int L = P * P;
    for (int w = tid; w < ne * L; w += nt) {
        const int e = w / L;
        const int l = w - e * L;
        const int j = l / P;
        const int kk = l - j * P;
        const BoxLine<WB, 0> la(e, j, kk);
        V x[Q], y[P];
#pragma unroll
        for (int n = 0; n < Q; ++n) x[n] = in[la(n)];
        eor_line<Eng, Q, P, +1>(x, y, m);
        typename Eng::S* dst = v + e * (P * P * P) + j * P + kk;
#pragma unroll
        for (int o = 0; o < P; ++o) dst[o * P * P] = Eng::store(y[o]);
    }
}

// One pass over the lines along k (thread per (i, j) line of every element)
// of a padded box holding (Q, Q, P): the line's P values are read once and
// `f(e, i, j, x, la)` computes and writes from registers (la: the line's
// addresses, for the other boxes' values on the same line).  The fused
// k-direction steps of BK1 and BK3 use it.
template <class Eng, class WB, int Q, int P, class F>
__device__ __forceinline__ void kline_pass(const typename Eng::V* in, int ne, int tid, int nt, F f)
{
    using V = typename Eng::V;
    constexpr int L = Q * Q;
    for (int w = tid; w < ne * L; w += nt) {
        const int e = w / L;
        const int l = w - e * L;
        const int i = l / Q;
        const int j = l - i * Q;
        const BoxLine<WB, 2> la(e, i, j);
        V x[P];
        line_load<WB, P>(in, la, x);
        f(e, i, j, x, la);
    }
}

// Dense (X, Y, Z) slice of S values of `ne` elements (element stride estride)
// -> padded work box, converted to the working type.
template <class Eng, class WB, int X, int Y, int Z>
__device__ __forceinline__ void load_box(const typename Eng::S* src, int estride, typename Eng::V* dst, int ne,
                                         int tid, int nt)
{
    constexpr int N = X * Y * Z;
    for (int w = tid; w < ne * N; w += nt) {
        const int e = w / N;
        const int x = w - e * N;
        const int i = x / (Y * Z);
        const int r = x - i * (Y * Z);
        const int j = r / Z;
        const int k = r - j * Z;
        dst[e * WB::size + WB::at(i, j, k)] = Eng::load(src[e * estride + x]);
    }
}

// A pass over the points of `ne` (X, Y, Z) boxes by lines along the first
// index: one thread per (e, j, k), f(e, j, k, d, b) called with the line's
// first dense offset d (e*X*Y*Z + j*Z + k) and its first work-box offset b; the
// callback walks the X points at the compile-time offsets d + i*Y*Z and
// b + i*WB::PS.  Consecutive threads take consecutive (j, k), so at each i
// a warp touches what the flat walk's warp touches, but the index arithmetic
// is paid once per line instead of once per point (the flat walk divides
// the point index by Q^3, Q^2 and Q at every point).
template <class WB, int X, int Y, int Z, class F>
__device__ __forceinline__ void ilines(int ne, int tid, int nt, F f)
{
    constexpr int YZ = Y * Z;
    for (int l = tid; l < ne * YZ; l += nt) {
        const int e = l / YZ;
        const int r = l - e * YZ;
        const int j = r / Z;
        const int k = r - j * Z;
        f(e, j, k, e * (X * YZ) + r, e * WB::size + WB::at(0, j, k));
    }
}

// The points n0, n0 + NS, n0 + 2 NS, ... (< Q) of one line, f(n) for each:
// NS = 1 walks the whole line at compile-time n; with NS > 1 (a line split
// among NS thread groups, n0 the group) the offsets n * stride are the
// per-line n0 * stride plus compile-time multiples.
template <int Q, int NS, class F>
__device__ __forceinline__ void line_points(const int n0, F f)
{
#pragma unroll
    for (int m = 0; m < (Q + NS - 1) / NS; ++m) {
        if (NS == 1) {
            f(m);
        } else {
            const int n = n0 + m * NS;
            if (n < Q) f(n);
        }
    }
}

// Padded work box -> dense (X, Y, Z) S values.
template <class Eng, class WB, int X, int Y, int Z>
__device__ __forceinline__ void store_box(const typename Eng::V* src, typename Eng::S* dst, int estride, int ne,
                                          int tid, int nt)
{
    constexpr int N = X * Y * Z;
    for (int w = tid; w < ne * N; w += nt) {
        const int e = w / N;
        const int x = w - e * N;
        const int i = x / (Y * Z);
        const int r = x - i * (Y * Z);
        const int j = r / Z;
        const int k = r - j * Z;
        dst[e * estride + x] = Eng::store(src[e * WB::size + WB::at(i, j, k)]);
    }
}

// Waits (bounded) for the batch's staged copies; the block agrees on the
// outcome with one barrier.  On a timeout the status word records
// BK_ERR_TIMEOUT, every thread waits once more (bounded) so that copies still
// in flight land before the block leaves, and true is returned: the caller
// returns without touching the batch.
__device__ __forceinline__ bool batch_wait_failed(uint64_t* bar, uint32_t phase, const DevCtx& ctx, int tid)
{
    const bool ok = mbar_wait_bounded(bar, phase, ctx.wait_limit);
    if (__syncthreads_or(ok ? 0 : 1)) {
        if (tid == 0) set_status(ctx, BK_ERR_TIMEOUT);
        if (!ok) mbar_wait_bounded(bar, phase, ctx.wait_limit);
        return true;
    }
    return false;
}

// ---- kernel parameters ---------------------------------------------------------

template <class C, int Q>
struct P5 {
    C D[Q * Q];          // D(i, n) = D[i*Q + n]
    EOMat<C, Q> eo;      // even-odd form of D (used when the kernel's EO is set)
    EOMat<C, Q> eot;     // even-odd form of D^T
};

template <class C, int Q>
struct P13 {
    C B[(Q - 1) * Q];   // B(i, p) = B[i*Q + p]
    C D[Q * Q];         // BK3: D(n, p) = D[n*Q + p]
    // even-odd forms (used when the kernel's EO is set): interpolation
    // M(p, i) = B(i, p) and its transpose, gradient M(p, n) = D(n, p) and its
    // transpose
    EORMat<C, Q, Q - 1> bi;
    EORMat<C, Q - 1, Q> bb;
    EORMat<C, Q, Q> dg;
    EORMat<C, Q, Q> dtr;
};

// Host: the even-odd forms of P13; true if B is centro-symmetric and D
// centro-antisymmetric (point sets symmetric about 0).
template <class C, int Q, class Conv>
inline bool make_p13_eo(P13<C, Q>& p, const double* B, const double* D, Conv conv)
{
    bool ok = make_eor<C, Q, Q - 1>(B, Q, true, +1, p.bi, conv);
    ok = make_eor<C, Q - 1, Q>(B, Q, false, +1, p.bb, conv) && ok;
    ok = make_eor<C, Q, Q>(D, Q, true, -1, p.dg, conv) && ok;
    ok = make_eor<C, Q, Q>(D, Q, false, -1, p.dtr, conv) && ok;
    return ok;
}

// ---- BK5 -----------------------------------------------------------------------

// Index of factor f at point (i, j, k) within an element's G.
template <class Eng, int Q, int F, int LAYOUT>
__device__ __forceinline__ int g_index(int i, int j, int f, int k)
{
    if (LAYOUT == 0) return ((f * Q + i) * Q + j) * Q + k;
    if (LAYOUT == 1) return ((i * Q + j) * F + f) * Q + k;
    return ((f * Q + k) * Q + i) * Q + j;
}

// DPAR != 0: three thread groups, one direction each (bk5_sweep_batch), and
// a fourth work box.
template <class Eng, int Q, int EB, int F, int LAYOUT, int DPAR = 0>
struct BK5Cfg {
    using S = typename Eng::S;
    using V = typename Eng::V;
    using WB = WBox5<Q, V>;
    static constexpr int Q3 = Q * Q * Q;
    static constexpr int LINES = ((EB * Q * Q + 31) / 32) * 32;   // one direction, whole warps
    static constexpr int NT = DPAR ? 3 * LINES : (LINES < 64 ? 64 : LINES);
    static constexpr int NBOX = DPAR ? 4 : 3;
    static constexpr int U_BYTES = stage_bytes<S>(EB * Q3);
    static constexpr int G_BYTES = stage_bytes<S>(EB * F * Q3);
    static constexpr int STAGE_BYTES = U_BYTES + G_BYTES;
    static constexpr int W_BYTES = ((NBOX * EB * WB::size * int(sizeof(V)) + 15) / 16) * 16;
    static constexpr int SMEM = STAGE_BYTES + W_BYTES + 16;
};

// One batch of ne elements of order Q whose u (us, dense; shared or global
// memory) and G (gs, in LAYOUT; shared or global memory) are given.  Dp:
// D(i, n) in parameter space; eo, eot: the even-odd forms of D and D^T (used
// when EO).  W0..W3: padded work boxes of at least ne elements (W3 only
// when DPAR).  v is written at vb (global), the mass term read at mb (global
// or shared, may be NULL) with u at us.  DOT (FP32 storage): the thread's
// running sum of u . v over its points in *dot, each product exact (FMA) and
// the sum compensated (float-float: about 44 bits).  after_pw: called by every
// thread after the pointwise stage, when the G stage is no longer read (nor
// u, unless the mass term or dot reads it at the end).  Ends with a block
// barrier (after which the stages may be reused) unless end_sync is false.
// GS: the type G is stored in (the storage type, or float-float pairs split
// ahead of time).
//
// Stages: load u into a box; gradient (three sweeps); pointwise fluxes;
// transposed sweeps; last pass (sum of the three terms, mass term, store).
// Even-odd without DPAR (KFUSE): the transposed k sweep and the last pass
// are one pass over k lines in registers.
//
// DPAR (even-odd only): the three sweeps of a stage run at the same time on
// three thread groups of nt/3 threads, one direction per group (warp-uniform
// branches when nt/3 is a multiple of 32); qt goes to the fourth box.  Three
// times the threads per element at the same shared memory per element: the
// latency-bound float-float arithmetic gets more warps per SM.  DPAR = 1:
// one code body per direction (strides known at compile time); DPAR = 2: one
// body for all three, the direction's strides in registers (a third of the
// instruction footprint of the stage).
struct NoOp {
    __device__ __forceinline__ void operator()() const {}
};

template <class Eng, int Q, int F, int LAYOUT, bool EO, int DPAR = 0, class AfterPw = NoOp, bool DOT = false,
          class GS = typename Eng::S>
__device__ __forceinline__ void bk5_sweep_batch(const typename Eng::C* __restrict__ Dp,
                                                const EOMat<typename Eng::C, Q>& eo,
                                                const EOMat<typename Eng::C, Q>& eot, const typename Eng::S* us,
                                                const GS* gs, typename Eng::V* W0, typename Eng::V* W1,
                                                typename Eng::V* W2, typename Eng::V* W3, int ne, int tid, int nt,
                                                typename Eng::S* __restrict__ vb,
                                                const typename Eng::S* __restrict__ mb, double lambda,
                                                ffacc* dot = nullptr, AfterPw after_pw = AfterPw(),
                                                const bool end_sync = true)
{
    static_assert(!DOT || sizeof(typename Eng::S) == 4, "the fused dot product is for FP32 storage");
    static_assert(!DPAR || EO, "direction-parallel sweeps need the even-odd form");
    using S = typename Eng::S;
    using V = typename Eng::V;
    using A = typename Eng::A;
    using WB = WBox5<Q, V>;
    constexpr int Q3 = Q * Q * Q;
    const Mat<typename Eng::C, Q, false> Dm{Dp};   // D(i, n)
    const Mat<typename Eng::C, Q, true> Dt{Dp};    // D(n, i)
    const S lam = S(lambda);
    // the k-direction transposed sweep fused into the last pass (even-odd,
    // one thread per line): one write and one read of the box fewer and one
    // barrier less (BK5 mixed q = 6, interleaved G: 113 -> 126 GDoF/s; the
    // Helmholtz launch 100 -> 107).  Not for FP32 storage at Q = 8, where
    // the apply runs at the HBM roofline and a thread's Q consecutive stores
    // (strided across the warp) cost more than the traffic saved (199 -> 190)
    constexpr bool KFUSE = EO && DPAR == 0 && !(sizeof(S) == 4 && Q == 8);
    // thread group of the direction-parallel stages
    const int ntd = DPAR ? nt / 3 : nt;
    const int grp = DPAR ? tid / ntd : 0;
    const int tg = tid - grp * ntd;
    V* QT = DPAR ? W3 : W2;   // qt, and the third transposed term
    // The per-point passes (load, fluxes, last pass) go by lines, the points
    // of a line at compile-time offsets from its base (ilines, line_points):
    // one thread per line, or in the direction-parallel blocks each line
    // split among the three groups (group g takes the points g, g + 3, ..).
    // A split of Q = 3m + 1 points gives one group a point more than the
    // others (float-float p = 6, q = 7: 32.6 -> 31.2 GDoF/s when tried), so
    // those blocks walk the points flat (point w of the batch, its indices
    // by division), which spreads them evenly over all threads.
    constexpr bool FLAT = DPAR != 0 && Q % 3 == 1;
    constexpr int LS = DPAR ? 3 : 1;
    const int lt = DPAR ? tg : tid;     // the thread's first line
    const int lnt = DPAR ? ntd : nt;    // threads per line set
    const int ln0 = DPAR ? grp : 0;     // the thread's first point of a line
    const bool lact = !DPAR || grp < 3;
    // 2. u -> W2 (working type, padded)
    if constexpr (FLAT) {
        load_box<Eng, WB, Q, Q, Q>(us, Q3, W2, ne, tid, nt);
    } else if (lact) {
        ilines<WB, Q, Q, Q>(ne, lt, lnt, [&](int, int, int, int d, int b) {
            line_points<Q, LS>(ln0, [&](int i) { W2[b + i * WB::PS] = Eng::load(us[d + i * Q * Q]); });
        });
    }
    __syncthreads();
    // 3. gradient: qr -> W0 (along i), qs -> W1 (along j), qt (along k) ->
    //    QT (in place into W2 after the other two have read it unless DPAR)
    if constexpr (DPAR == 2) {
        if (grp < 3) sweep_eo_dyn<Eng, WB, Q>(W2, grp == 0 ? W0 : (grp == 1 ? W1 : W3), ne, eo, tg, ntd, grp);
    } else if constexpr (DPAR == 1) {
        if (grp == 0) sweep_eo<Eng, WB, 0, Q>(W2, W0, ne, eo, tg, ntd);
        else if (grp == 1) sweep_eo<Eng, WB, 1, Q>(W2, W1, ne, eo, tg, ntd);
        else if (grp == 2) sweep_eo<Eng, WB, 2, Q>(W2, W3, ne, eo, tg, ntd);
    } else if constexpr (EO) {
        sweep_eo<Eng, WB, 0, Q>(W2, W0, ne, eo, tid, nt);
        sweep_eo<Eng, WB, 1, Q>(W2, W1, ne, eo, tid, nt);
        __syncthreads();
        sweep_eo<Eng, WB, 2, Q>(W2, W2, ne, eo, tid, nt);
    } else {
        sweep<Eng, WB, 0, Q, Q, Q, Q>(W2, W0, ne, Dm, tid, nt);
        sweep<Eng, WB, 1, Q, Q, Q, Q>(W2, W1, ne, Dm, tid, nt);
        __syncthreads();
        sweep<Eng, WB, 2, Q, Q, Q, Q>(W2, W2, ne, Dm, tid, nt);
    }
    __syncthreads();
    // 4. fluxes with the symmetric (F = 6) or full (F = 9) factors
    //    (point wi of the boxes, g(f) the point's factor f)
    auto flux = [&](const int wi, auto g) {
        const V qr = W0[wi], qs = W1[wi], qt = QT[wi];
        A r0, r1, r2;
        if (F == 6) {
            const V g0 = g(0), g1 = g(1), g2 = g(2), g3 = g(3), g4 = g(4), g5 = g(5);
            r0 = Eng::vfirst(g0, qr); Eng::vmadd(r0, g1, qs); Eng::vmadd(r0, g2, qt);
            r1 = Eng::vfirst(g1, qr); Eng::vmadd(r1, g3, qs); Eng::vmadd(r1, g4, qt);
            r2 = Eng::vfirst(g2, qr); Eng::vmadd(r2, g4, qs); Eng::vmadd(r2, g5, qt);
        } else {
            r0 = Eng::vfirst(g(0), qr); Eng::vmadd(r0, g(1), qs); Eng::vmadd(r0, g(2), qt);
            r1 = Eng::vfirst(g(3), qr); Eng::vmadd(r1, g(4), qs); Eng::vmadd(r1, g(5), qt);
            r2 = Eng::vfirst(g(6), qr); Eng::vmadd(r2, g(7), qs); Eng::vmadd(r2, g(8), qt);
        }
        W0[wi] = Eng::result(r0);
        W1[wi] = Eng::result(r1);
        QT[wi] = Eng::result(r2);
    };
    if constexpr (FLAT) {
        for (int w = tid; w < ne * Q3; w += nt) {
            const int e = w / Q3;
            const int x = w - e * Q3;
            int i, j, k;
            if (LAYOUT == 2) {   // walk points in G's (k, i, j) order
                k = x / (Q * Q);
                i = (x / Q) % Q;
                j = x % Q;
            } else {
                i = x / (Q * Q);
                j = (x / Q) % Q;
                k = x % Q;
            }
            const GS* ge = gs + e * F * Q3;
            flux(e * WB::size + WB::at(i, j, k),
                 [&](int f) { return Eng::load(ge[g_index<Eng, Q, F, LAYOUT>(i, j, f, k)]); });
        }
    } else if (lact) {
        if constexpr (LAYOUT == 2) {
            // lines along k, one per (e, i, j): G(e, f, k, i, j) of
            // consecutive threads is consecutive
            for (int l = lt; l < ne * Q * Q; l += lnt) {
                const int e = l / (Q * Q);
                const int r = l - e * (Q * Q);   // i*Q + j
                const int i = r / Q;
                const int j = r - i * Q;
                const int wb = e * WB::size + WB::at(i, j, 0);
                const GS* ge = gs + e * F * Q3 + r;
                line_points<Q, LS>(ln0, [&](int k) {
                    flux(wb + k, [&](int f) { return Eng::load(ge[(f * Q + k) * Q * Q]); });
                });
            }
        } else {
            // lines along i, one per (e, j, k)
            ilines<WB, Q, Q, Q>(ne, lt, lnt, [&](int e, int j, int k, int, int b) {
                const GS* ge = gs + e * F * Q3;
                line_points<Q, LS>(ln0, [&](int i) {
                    flux(b + i * WB::PS,
                         [&](int f) { return Eng::load(ge[g_index<Eng, Q, F, LAYOUT>(i, j, f, k)]); });
                });
            });
        }
    }
    __syncthreads();
    after_pw();   // the G stage (and u, without a mass term) is free from here
    // 5. transposed derivatives, in place: along i on W0, along j on W1 and
    //    (even-odd) along k on QT
    if constexpr (DPAR == 2) {
        if (grp < 3) {
            // summed in the last pass, never multiplied: loose pairs
            V* Wg = grp == 0 ? W0 : (grp == 1 ? W1 : W3);
            sweep_eo_dyn<Eng, WB, Q, true>(Wg, Wg, ne, eot, tg, ntd, grp);
        }
    } else if constexpr (DPAR == 1) {
        if (grp == 0) sweep_eo<Eng, WB, 0, Q, true>(W0, W0, ne, eot, tg, ntd);
        else if (grp == 1) sweep_eo<Eng, WB, 1, Q, true>(W1, W1, ne, eot, tg, ntd);
        else if (grp == 2) sweep_eo<Eng, WB, 2, Q, true>(W3, W3, ne, eot, tg, ntd);
    } else if constexpr (EO) {
        // summed in the last pass, never multiplied: loose pairs
        sweep_eo<Eng, WB, 0, Q, true>(W0, W0, ne, eot, tid, nt);
        sweep_eo<Eng, WB, 1, Q, true>(W1, W1, ne, eot, tid, nt);
        // the k direction: in registers in the last pass (KFUSE, below), or
        // here
        if constexpr (!KFUSE) sweep_eo<Eng, WB, 2, Q, true>(W2, W2, ne, eot, tid, nt);
    } else {
        sweep<Eng, WB, 0, Q, Q, Q, Q>(W0, W0, ne, Dt, tid, nt);
        sweep<Eng, WB, 1, Q, Q, Q, Q>(W1, W1, ne, Dt, tid, nt);
    }
    __syncthreads();
    if constexpr (!EO) {
        // 6. along k on W2 plus the other two terms, back into W2 (each line
        //    is read completely before it is written; lines are disjoint)
        constexpr int L = Q * Q;
        for (int w = tid; w < ne * L; w += nt) {
            const int e = w / L;
            const int l = w - e * L;
            const int i = l / Q;
            const int j = l - i * Q;
            const BoxLine<WB, 2> la(e, i, j);
            V x[Q];
#pragma unroll
            for (int n = 0; n < Q; ++n) x[n] = W2[la(n)];
#pragma unroll
            for (int o = 0; o < Q; ++o) {
                A acc = Eng::first(Dt(o, 0), x[0]);
#pragma unroll
                for (int n = 1; n < Q; ++n) Eng::madd(acc, Dt(o, n), x[n]);
                V res;
                if constexpr (HasSum3<Eng>::value) {
                    res = Eng::sum3(Eng::result(acc), W0[la(o)], W1[la(o)]);
                } else {
                    Eng::add(acc, W0[la(o)]);
                    Eng::add(acc, W1[la(o)]);
                    res = Eng::loose(acc);
                }
                W2[la(o)] = res;
            }
        }
        __syncthreads();
    }
    // 7. -> v in global memory (consecutive threads, consecutive values):
    //    the sum of the three terms (even-odd: here; otherwise already in W2)
    //    and the Helmholtz mass term lambda * mass * u in the storage type's
    //    arithmetic (double for the FP64 engines).  The loop is written twice
    //    (with and without the mass term) so that no point carries the
    //    predicated-off mass arithmetic.
    auto last_point = [&](auto with_mass, const int w, const int wi) {
        V res;
        if constexpr (EO) {
            if constexpr (HasSum3<Eng>::value) {
                res = Eng::sum3(QT[wi], W0[wi], W1[wi]);
            } else {
                A acc = Eng::from(QT[wi]);
                Eng::add(acc, W0[wi]);
                Eng::add(acc, W1[wi]);
                res = Eng::loose(acc);   // store() renormalises
            }
        } else {
            res = W2[wi];
        }
        S out = Eng::store(res);
        if constexpr (decltype(with_mass)::value) out += lam * mb[w] * us[w];
        vb[w] = out;
        if constexpr (DOT) acc_madd_f(*dot, us[w], out);   // u . A u for CG, compensated
    };
    auto last_pass = [&](auto with_mass) {
        if constexpr (FLAT) {
            for (int w = tid; w < ne * Q3; w += nt) {
                const int e = w / Q3;
                const int x = w - e * Q3;
                const int i = x / (Q * Q);
                const int j = (x / Q) % Q;
                const int k = x % Q;
                last_point(with_mass, w, e * WB::size + WB::at(i, j, k));
            }
        } else if (lact) {
            ilines<WB, Q, Q, Q>(ne, lt, lnt, [&](int, int, int, int d, int b) {
                line_points<Q, LS>(ln0, [&](int i) { last_point(with_mass, d + i * Q * Q, b + i * WB::PS); });
            });
        }
    };
    // 7'. (KFUSE) one thread per k line: the transposed k-derivative of the
    //    third flux in registers (no write and re-read of the box), the sum,
    //    the mass term, each thread storing its line's Q values
    auto kline_last = [&](auto with_mass) {
        kline_pass<Eng, WB, Q, Q>(QT, ne, tid, nt, [&](int e, int i, int j, const V (&x)[Q], const BoxLine<WB, 2>& la) {
            V t[Q];
            eo_line<Eng, Q, true>(x, t, eot);   // summed next: loose pairs
            const int w0 = e * Q3 + (i * Q + j) * Q;
#pragma unroll
            for (int o = 0; o < Q; ++o) {
                V res;
                if constexpr (HasSum3<Eng>::value) {
                    res = Eng::sum3(t[o], W0[la(o)], W1[la(o)]);
                } else {
                    A acc = Eng::from(t[o]);
                    Eng::add(acc, W0[la(o)]);
                    Eng::add(acc, W1[la(o)]);
                    res = Eng::loose(acc);   // store() renormalises
                }
                S out = Eng::store(res);
                if constexpr (decltype(with_mass)::value) out += lam * mb[w0 + o] * us[w0 + o];
                vb[w0 + o] = out;
                if constexpr (DOT) acc_madd_f(*dot, us[w0 + o], out);
            }
        });
    };
    if constexpr (KFUSE) {
        if (mb != nullptr)
            kline_last(std::true_type{});
        else
            kline_last(std::false_type{});
    } else {
        if (mb != nullptr)
            last_pass(std::true_type{});
        else
            last_pass(std::false_type{});
    }
    // end_sync (uniform): false when the caller's next step is a block
    // barrier anyway and nothing before it writes what the last pass read
    if (end_sync) __syncthreads();
}

// The block walks batches bt = blockIdx.x, + gridDim.x, ...  One stage buffer:
// the next batch's u and G are copied into it as soon as the current batch
// stops reading them (after the pointwise stage; u after the last pass when a
// mass term reads it there), so the copies overlap the transposed sweeps and
// the last pass instead of stalling the block at the start of each batch.
template <class Eng, int Q, int EB, int F, int LAYOUT, bool EO = false, int DPAR = 0, class GS = typename Eng::S>
__global__ void __launch_bounds__(BK5Cfg<Eng, Q, EB, F, LAYOUT, DPAR>::NT)
    bk5_kernel(const __grid_constant__ P5<typename Eng::C, Q> prm, const long long E,
               const typename Eng::S* __restrict__ u, const GS* __restrict__ G,
               const typename Eng::S* __restrict__ mass, const double lambda, typename Eng::S* __restrict__ v,
               const DevCtx ctx)
{
    using Cfg = BK5Cfg<Eng, Q, EB, F, LAYOUT, DPAR>;
    using S = typename Eng::S;
    using V = typename Eng::V;
    using WB = typename Cfg::WB;
    static_assert(sizeof(GS) == sizeof(S), "G is staged in the footprint of the storage type");
    constexpr int Q3 = Cfg::Q3;
    extern __shared__ __align__(16) unsigned char smem[];
    V* W0 = reinterpret_cast<V*>(smem + Cfg::STAGE_BYTES);
    V* W1 = W0 + EB * WB::size;
    V* W2 = W1 + EB * WB::size;
    V* W3 = DPAR ? W2 + EB * WB::size : nullptr;
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem + Cfg::STAGE_BYTES + Cfg::W_BYTES);
    const int tid = threadIdx.x;
    const int nt = Cfg::NT;

    if (tid == 0) {
        mbar_init(bar, 1);
        fence_mbar_init();
    }
    __syncthreads();
    const long long nbatch = (E + EB - 1) / EB;
    // where the staged batch's u and G landed
    const S* us = nullptr;
    const GS* gs = nullptr;
    // 1. stage G (every thread; thread 0 issues the TMA part and adds its
    //    bytes to the phase without arriving), then u (thread 0 arrives):
    //    batch bt's phase completes when both have landed
    auto issue_g = [&](long long bt) {
        const long long e0 = bt * EB;
        const int ne = int((E - e0) < EB ? (E - e0) : EB);
        uint32_t tx = 0;
        if (tid == 0) fence_proxy_async();
        gs = stage_issue<GS>(smem + Cfg::U_BYTES, G + e0 * F * Q3, ne * F * Q3, G + E * F * Q3, bar, tx, tid, nt);
        if (tid == 0) mbar_expect_tx(bar, tx);
    };
    auto issue_u = [&](long long bt) {
        const long long e0 = bt * EB;
        const int ne = int((E - e0) < EB ? (E - e0) : EB);
        uint32_t tx = 0;
        if (tid == 0) fence_proxy_async();
        us = stage_issue<S>(smem, u + e0 * Q3, ne * Q3, u + E * Q3, bar, tx, tid, nt);
        if (tid == 0) mbar_arrive_expect_tx(bar, tx);
    };
    if (blockIdx.x < nbatch) {
        issue_g(blockIdx.x);
        issue_u(blockIdx.x);
    }
    uint32_t phase = 0;
    for (long long bt = blockIdx.x; bt < nbatch; bt += gridDim.x, phase ^= 1u) {
        if (batch_wait_failed(bar, phase, ctx, tid)) return;
        const long long e0 = bt * EB;
        const int ne = int((E - e0) < EB ? (E - e0) : EB);
        const long long next = bt + gridDim.x;
        const S* mb = (mass != nullptr) ? mass + e0 * Q3 : nullptr;
        const S* ub = us;
        const GS* gb = gs;
        // after the pointwise stage the G stage is free, and the u stage too
        // unless the mass term reads u in the last pass (then u follows the
        // batch)
        auto early = [&]() {
            if (next < nbatch) {
                issue_g(next);
                if (mass == nullptr) issue_u(next);
            }
        };
        // the next batch's wait ends with a block barrier before anything
        // writes the boxes or the stage again, except the copy of u that
        // follows a batch with the mass term (its last pass reads u): only
        // that batch ends with its own barrier
        bk5_sweep_batch<Eng, Q, F, LAYOUT, EO, DPAR>(prm.D, prm.eo, prm.eot, ub, gb, W0, W1, W2, W3, ne, tid, nt,
                                                     v + e0 * Q3, mb, lambda, nullptr, early, mass != nullptr);
        if (mass != nullptr && next < nbatch) issue_u(next);
    }
}

// ---- BK1 -----------------------------------------------------------------------

template <class Eng, int Q, int EB>
struct BK1Cfg {
    using S = typename Eng::S;
    using V = typename Eng::V;
    using WB = WBox3<Q, V>;
    static constexpr int P = Q - 1;
    static constexpr int Q3 = Q * Q * Q;
    static constexpr int P3 = P * P * P;
    static constexpr int NT = ((EB * Q * Q + 31) / 32) * 32 < 64 ? 64 : ((EB * Q * Q + 31) / 32) * 32;
    static constexpr int U_BYTES = stage_bytes<S>(EB * Q3);   // also holds the P^3 output
    static constexpr int J_BYTES = stage_bytes<S>(EB * Q3);
    static constexpr int W_BYTES = ((2 * EB * WB::size * int(sizeof(V)) + 15) / 16) * 16;
    static constexpr int SMEM = U_BYTES + J_BYTES + W_BYTES + 16;
};

template <class Eng, int Q, int EB, bool EO = false>
__global__ void __launch_bounds__(BK1Cfg<Eng, Q, EB>::NT)
    bk1_kernel(const __grid_constant__ P13<typename Eng::C, Q> prm, const long long E,
               const typename Eng::S* __restrict__ u, const typename Eng::S* __restrict__ jxw, const int jxw_t,
               typename Eng::S* __restrict__ v, const DevCtx ctx)
{
    using Cfg = BK1Cfg<Eng, Q, EB>;
    using S = typename Eng::S;
    using V = typename Eng::V;
    using WB = typename Cfg::WB;
    constexpr int P = Cfg::P, Q3 = Cfg::Q3, P3 = Cfg::P3;
    // u and v straight between the stage / HBM and the first / last
    // interpolation when they need no conversion; the float-float engine's
    // split and join are spread over all threads by the load and store passes
    // instead (in the line passes a quarter of the threads would do them)
    constexpr bool kDirectIO = std::is_same<S, V>::value;
    extern __shared__ __align__(16) unsigned char smem[];
    unsigned char* ustage = smem;
    unsigned char* jstage = ustage + Cfg::U_BYTES;
    V* W0 = reinterpret_cast<V*>(jstage + Cfg::J_BYTES);
    V* W1 = W0 + EB * WB::size;
    uint64_t* bar = reinterpret_cast<uint64_t*>(jstage + Cfg::J_BYTES + Cfg::W_BYTES);
    const int tid = threadIdx.x;
    const int nt = Cfg::NT;
    // interpolation out(p) = sum_i in(i) B(i, p): M(o=p, n=i) = B[i*Q + p]
    const Mat<typename Eng::C, Q, true> Bi{prm.B};
    // back: out(i) = sum_p in(p) B(i, p): M(o=i, n=p) = B[i*Q + p]
    const Mat<typename Eng::C, Q, false> Bb{prm.B};

    if (tid == 0) {
        mbar_init(bar, 1);
        fence_mbar_init();
    }
    __syncthreads();
    const long long nbatch = (E + EB - 1) / EB;
    // u and qdata of batch bt into the stage; the next batch is issued as
    // soon as the pointwise stage has read it (copies overlap the sweeps back)
    const S* us = nullptr;
    const S* js = nullptr;
    auto issue = [&](long long bt) {
        const long long e0 = bt * EB;
        const int ne = int((E - e0) < EB ? (E - e0) : EB);
        uint32_t tx = 0;
        if (tid == 0) fence_proxy_async();
        us = stage_issue<S>(ustage, u + e0 * P3, ne * P3, u + E * P3, bar, tx, tid, nt);
        js = stage_issue<S>(jstage, jxw + e0 * Q3, ne * Q3, jxw + E * Q3, bar, tx, tid, nt);
        if (tid == 0) mbar_arrive_expect_tx(bar, tx);
    };
    if (blockIdx.x < nbatch) issue(blockIdx.x);
    uint32_t phase = 0;
    for (long long bt = blockIdx.x; bt < nbatch; bt += gridDim.x, phase ^= 1u) {
        const long long e0 = bt * EB;
        const int ne = int((E - e0) < EB ? (E - e0) : EB);
        if (batch_wait_failed(bar, phase, ctx, tid)) return;
        if constexpr (EO) {   // B centro-symmetric (GLL nodes, Gauss points)
            if constexpr (kDirectIO) {
                interp0_from_dense<Eng, WB, P, Q>(us, W1, ne, prm.bi, tid, nt);    // (Q,P,P)
            } else {
                load_box<Eng, WB, P, P, P>(us, P3, W0, ne, tid, nt);
                __syncthreads();
                sweep_eor<Eng, WB, 0, P, P, P, Q, +1>(W0, W1, ne, prm.bi, tid, nt);   // (Q,P,P)
            }
            __syncthreads();
            sweep_eor<Eng, WB, 1, Q, P, P, Q, +1>(W1, W0, ne, prm.bi, tid, nt);   // (Q,Q,P)
            __syncthreads();
            // along k in registers: interpolate to the points, times JxW,
            // back to the nodes, (Q,Q,P) in place
            kline_pass<Eng, WB, Q, P>(W0, ne, tid, nt, [&](int e, int i, int j, const V (&x)[P], const BoxLine<WB, 2>& la) {
                V y[Q], z[P];
                eor_line<Eng, P, Q, +1>(x, y, prm.bi);
                // point (i, j, o) of JxW(e,p,q,r), or of JxW_t(e,r,q,p)
                if (jxw_t) {
                    const S* jl = js + e * Q3 + j * Q + i;
#pragma unroll
                    for (int o = 0; o < Q; ++o) y[o] = Eng::mul(y[o], Eng::load(jl[o * Q * Q]));
                } else {
                    const S* jl = js + e * Q3 + (i * Q + j) * Q;
#pragma unroll
                    for (int o = 0; o < Q; ++o) y[o] = Eng::mul(y[o], Eng::load(jl[o]));
                }
                eor_line<Eng, Q, P, +1>(y, z, prm.bb);
#pragma unroll
                for (int o = 0; o < P; ++o) W0[la(o)] = z[o];
            });
            __syncthreads();
            if (bt + gridDim.x < nbatch) issue(bt + gridDim.x);   // the stage is free
            sweep_eor<Eng, WB, 1, Q, Q, P, P, +1>(W0, W1, ne, prm.bb, tid, nt);   // (Q,P,P)
            __syncthreads();
            if constexpr (kDirectIO) {
                interp0_to_dense<Eng, WB, P, Q>(W1, v + e0 * P3, ne, prm.bb, tid, nt);  // -> v
            } else {
                sweep_eor<Eng, WB, 0, Q, P, P, P, +1, true>(W1, W0, ne, prm.bb, tid, nt);   // (P,P,P), stored next
                __syncthreads();
                store_box<Eng, WB, P, P, P>(W0, v + e0 * P3, P3, ne, tid, nt);
            }
            __syncthreads();
        } else {
            load_box<Eng, WB, P, P, P>(us, P3, W0, ne, tid, nt);
            __syncthreads();
            sweep<Eng, WB, 0, P, P, P, Q>(W0, W1, ne, Bi, tid, nt);   // (Q,P,P)
            __syncthreads();
            sweep<Eng, WB, 1, Q, P, P, Q>(W1, W0, ne, Bi, tid, nt);   // (Q,Q,P)
            __syncthreads();
            sweep<Eng, WB, 2, Q, Q, P, Q>(W0, W1, ne, Bi, tid, nt);   // (Q,Q,Q)
            __syncthreads();
            for (int w = tid; w < ne * Q3; w += nt) {
                const int e = w / Q3;
                const int x = w - e * Q3;
                const int i = x / (Q * Q), j = (x / Q) % Q, k = x % Q;
                const int wi = e * WB::size + WB::at(i, j, k);
                const int jx = jxw_t ? (k * Q + j) * Q + i : x;
                W1[wi] = Eng::mul(W1[wi], Eng::load(js[e * Q3 + jx]));
            }
            __syncthreads();
            if (bt + gridDim.x < nbatch) issue(bt + gridDim.x);   // the stage is free
            sweep<Eng, WB, 2, Q, Q, Q, P>(W1, W0, ne, Bb, tid, nt);   // (Q,Q,P)
            __syncthreads();
            sweep<Eng, WB, 1, Q, Q, P, P>(W0, W1, ne, Bb, tid, nt);   // (Q,P,P)
            __syncthreads();
            sweep<Eng, WB, 0, Q, P, P, P>(W1, W0, ne, Bb, tid, nt);   // (P,P,P)
            __syncthreads();
            // padded box -> v (consecutive threads, consecutive values)
            store_box<Eng, WB, P, P, P>(W0, v + e0 * P3, P3, ne, tid, nt);
            __syncthreads();
        }
    }
}

// ---- BK3 -----------------------------------------------------------------------

// DPAR != 0: three thread groups run the three gradient sweeps and the three
// transposed ones at the same time (one shared code body); the other stages
// use all threads.
template <class Eng, int Q, int EB, int DPAR = 0>
struct BK3Cfg {
    using S = typename Eng::S;
    using V = typename Eng::V;
    using WB = WBox3<Q, V, true>;   // swizzled rows at 4-byte Q = 8 (bk3_swz)
    static constexpr int P = Q - 1;
    static constexpr int Q3 = Q * Q * Q;
    static constexpr int P3 = P * P * P;
    static constexpr int LINES = ((EB * Q * Q + 31) / 32) * 32;
    static constexpr int NT = DPAR ? 3 * LINES : (LINES < 64 ? 64 : LINES);
    static constexpr int U_BYTES = stage_bytes<S>(EB * P3);
    static constexpr int G_BYTES = stage_bytes<S>(EB * 6 * Q3);
    static constexpr int K_BYTES = stage_bytes<S>(EB * Q3);
    static constexpr int W_BYTES = ((4 * EB * WB::size * int(sizeof(V)) + 15) / 16) * 16;
    static constexpr int SMEM = U_BYTES + G_BYTES + K_BYTES + W_BYTES + 16;
};

template <class Eng, int Q, int EB, bool EO = false, int DPAR = 0, class GS = typename Eng::S>
__global__ void __launch_bounds__(BK3Cfg<Eng, Q, EB, DPAR>::NT)
    bk3_kernel(const __grid_constant__ P13<typename Eng::C, Q> prm, const long long E,
               const typename Eng::S* __restrict__ u, const GS* __restrict__ G,
               const typename Eng::S* __restrict__ kq, typename Eng::S* __restrict__ v, const DevCtx ctx)
{
    static_assert(!DPAR || EO, "direction-parallel sweeps need the even-odd form");
    using Cfg = BK3Cfg<Eng, Q, EB, DPAR>;
    using S = typename Eng::S;
    static_assert(sizeof(GS) == sizeof(S), "G is staged in the footprint of the storage type");
    using V = typename Eng::V;
    using A = typename Eng::A;
    using WB = typename Cfg::WB;
    constexpr int P = Cfg::P, Q3 = Cfg::Q3, P3 = Cfg::P3;
    // u and v straight between the stage / HBM and the first / last
    // interpolation when they need no conversion; the float-float engine's
    // split and join are spread over all threads by the load and store passes
    // instead (in the line passes a quarter of the threads would do them)
    constexpr bool kDirectIO = std::is_same<S, V>::value;
    extern __shared__ __align__(16) unsigned char smem[];
    unsigned char* ustage = smem;
    unsigned char* gstage = ustage + Cfg::U_BYTES;
    unsigned char* kstage = gstage + Cfg::G_BYTES;
    V* W0 = reinterpret_cast<V*>(kstage + Cfg::K_BYTES);
    V* W1 = W0 + EB * WB::size;
    V* W2 = W1 + EB * WB::size;
    V* W3 = W2 + EB * WB::size;
    uint64_t* bar = reinterpret_cast<uint64_t*>(kstage + Cfg::K_BYTES + Cfg::W_BYTES);
    const int tid = threadIdx.x;
    const int nt = Cfg::NT;
    const Mat<typename Eng::C, Q, true> Bi{prm.B};    // M(p, i) = B[i*Q + p]
    const Mat<typename Eng::C, Q, false> Bb{prm.B};   // M(i, p) = B[i*Q + p]
    const Mat<typename Eng::C, Q, true> Dg{prm.D};    // q(p) = sum_n u(n) D(n, p)
    const Mat<typename Eng::C, Q, false> Dtr{prm.D};  // sum_n f(n) D(p, n)

    if (tid == 0) {
        mbar_init(bar, 1);
        fence_mbar_init();
    }
    __syncthreads();
    const long long nbatch = (E + EB - 1) / EB;
    // u, G and k of batch bt into the stage (every thread; thread 0 issues
    // the TMA part and arrives).  The next batch is issued as soon as the
    // pointwise stage has read the stage, so its copies overlap the
    // transposed sweeps.
    const S* us = nullptr;
    const GS* gs = nullptr;
    const S* ks = nullptr;
    auto issue = [&](long long bt) {
        const long long e0 = bt * EB;
        const int ne = int((E - e0) < EB ? (E - e0) : EB);
        uint32_t tx = 0;
        if (tid == 0) fence_proxy_async();
        us = stage_issue<S>(ustage, u + e0 * P3, ne * P3, u + E * P3, bar, tx, tid, nt);
        gs = stage_issue<GS>(gstage, G + e0 * 6 * Q3, ne * 6 * Q3, G + E * 6 * Q3, bar, tx, tid, nt);
        ks = (kq != nullptr) ? stage_issue<S>(kstage, kq + e0 * Q3, ne * Q3, kq + E * Q3, bar, tx, tid, nt) : nullptr;
        if (tid == 0) mbar_arrive_expect_tx(bar, tx);
    };
    if (blockIdx.x < nbatch) issue(blockIdx.x);
    uint32_t phase = 0;
    for (long long bt = blockIdx.x; bt < nbatch; bt += gridDim.x, phase ^= 1u) {
        const long long e0 = bt * EB;
        const int ne = int((E - e0) < EB ? (E - e0) : EB);
        if (batch_wait_failed(bar, phase, ctx, tid)) return;
        // fluxes (k G grad u with the coefficient); written twice, with and
        // without k, so that no point carries predicated-off products
        auto fluxes = [&](auto with_k) {
            for (int w = tid; w < ne * Q3; w += nt) {
                const int e = w / Q3;
                const int x = w - e * Q3;
                const int i = x / (Q * Q), j = (x / Q) % Q, k = x % Q;
                const int wi = e * WB::size + WB::at(i, j, k);
                V qr = W0[wi], qs = W1[wi], qt = W3[wi];
                if constexpr (decltype(with_k)::value) {
                    const V kk = Eng::load(ks[e * Q3 + x]);
                    qr = Eng::mul(kk, qr);
                    qs = Eng::mul(kk, qs);
                    qt = Eng::mul(kk, qt);
                }
                const GS* ge = gs + e * 6 * Q3 + x;   // factor-major
                const V g0 = Eng::load(ge[0]), g1 = Eng::load(ge[Q3]), g2 = Eng::load(ge[2 * Q3]);
                const V g3 = Eng::load(ge[3 * Q3]), g4 = Eng::load(ge[4 * Q3]), g5 = Eng::load(ge[5 * Q3]);
                A r0 = Eng::vfirst(g0, qr), r1 = Eng::vfirst(g1, qr), r2 = Eng::vfirst(g2, qr);
                Eng::vmadd(r0, g1, qs); Eng::vmadd(r0, g2, qt);
                Eng::vmadd(r1, g3, qs); Eng::vmadd(r1, g4, qt);
                Eng::vmadd(r2, g4, qs); Eng::vmadd(r2, g5, qt);
                W0[wi] = Eng::result(r0);
                W1[wi] = Eng::result(r1);
                W3[wi] = Eng::result(r2);
            }
        };
        // the transposed k-direction derivative of the third flux plus the
        // other two terms, at one (i, j) line: s = D^T x + W0 + W1
        auto sum_line = [&](const V (&t)[Q], V (&sv)[Q], const BoxLine<WB, 2>& la) {
            if constexpr (WB::VEC) {
                V w0[Q], w1[Q];
                line_load<WB, Q>(W0, la, w0);
                line_load<WB, Q>(W1, la, w1);
#pragma unroll
                for (int o = 0; o < Q; ++o) {
                    if constexpr (HasSum3<Eng>::value) {
                        sv[o] = Eng::sum3(t[o], w0[o], w1[o]);
                    } else {
                        A acc = Eng::from(t[o]);
                        Eng::add(acc, w0[o]);
                        Eng::add(acc, w1[o]);
                        sv[o] = Eng::result(acc);
                    }
                }
                return;
            }
#pragma unroll
            for (int o = 0; o < Q; ++o) {
                if constexpr (HasSum3<Eng>::value) {
                    sv[o] = Eng::sum3(t[o], W0[la(o)], W1[la(o)]);
                } else {
                    A acc = Eng::from(t[o]);
                    Eng::add(acc, W0[la(o)]);
                    Eng::add(acc, W1[la(o)]);
                    sv[o] = Eng::result(acc);
                }
            }
        };
        if constexpr (EO) {
            // B centro-symmetric, D centro-antisymmetric (GLL nodes, Gauss
            // points).  u straight from the stage into the first
            // interpolation, v straight from the last one to HBM.
            if constexpr (kDirectIO) {
                interp0_from_dense<Eng, WB, P, Q>(us, W1, ne, prm.bi, tid, nt);    // (Q,P,P)
            } else {
                load_box<Eng, WB, P, P, P>(us, P3, W0, ne, tid, nt);
                __syncthreads();
                sweep_eor<Eng, WB, 0, P, P, P, Q, +1>(W0, W1, ne, prm.bi, tid, nt);   // (Q,P,P)
            }
            __syncthreads();
            sweep_eor<Eng, WB, 1, Q, P, P, Q, +1>(W1, W0, ne, prm.bi, tid, nt);   // (Q,Q,P)
            __syncthreads();
            if constexpr (DPAR) {
                sweep_eor<Eng, WB, 2, Q, Q, P, Q, +1>(W0, W2, ne, prm.bi, tid, nt);   // u at the points: W2
                __syncthreads();
                const int grp = tid / Cfg::LINES;
                if (grp < 3)
                    sweep_eo_dyn<Eng, WB, Q>(W2, grp == 0 ? W0 : (grp == 1 ? W1 : W3), ne, prm.dg,
                                             tid - grp * Cfg::LINES, Cfg::LINES, grp);   // qr, qs, qt
            } else {
                // along k in registers: u at the points (W2) and its
                // k-derivative qt (W3)
                kline_pass<Eng, WB, Q, P>(W0, ne, tid, nt, [&](int, int, int, const V (&x)[P], const BoxLine<WB, 2>& la) {
                    V y[Q], t[Q];
                    eor_line<Eng, P, Q, +1>(x, y, prm.bi);
                    eor_line<Eng, Q, Q, -1>(y, t, prm.dg);
                    line_store<WB, Q>(W2, la, y);
                    line_store<WB, Q>(W3, la, t);
                });
                __syncthreads();
                sweep_eor<Eng, WB, 0, Q, Q, Q, Q, -1>(W2, W0, ne, prm.dg, tid, nt);   // qr
                sweep_eor<Eng, WB, 1, Q, Q, Q, Q, -1>(W2, W1, ne, prm.dg, tid, nt);   // qs
            }
            __syncthreads();
            if (ks != nullptr)
                fluxes(std::true_type{});
            else
                fluxes(std::false_type{});
            __syncthreads();
            if (bt + gridDim.x < nbatch) issue(bt + gridDim.x);   // the stage is free
            if constexpr (DPAR) {
                const int grp = tid / Cfg::LINES;
                if (grp < 3) {
                    V* Wg = grp == 0 ? W0 : (grp == 1 ? W1 : W3);
                    // summed along k next, never multiplied: loose pairs
                    sweep_eo_dyn<Eng, WB, Q, true>(Wg, Wg, ne, prm.dtr, tid - grp * Cfg::LINES, Cfg::LINES, grp);
                }
                __syncthreads();
                // the three terms summed into W2, then back along k
                kline_pass<Eng, WB, Q, Q>(W3, ne, tid, nt, [&](int, int, int, const V (&x)[Q], const BoxLine<WB, 2>& la) {
                    V sv[Q];
                    sum_line(x, sv, la);
                    line_store<WB, Q>(W2, la, sv);
                });
                __syncthreads();
                sweep_eor<Eng, WB, 2, Q, Q, Q, P, +1>(W2, W0, ne, prm.bb, tid, nt);   // (Q,Q,P)
            } else {
                // summed along k next, never multiplied: loose pairs
                sweep_eor<Eng, WB, 0, Q, Q, Q, Q, -1, true>(W0, W0, ne, prm.dtr, tid, nt);
                sweep_eor<Eng, WB, 1, Q, Q, Q, Q, -1, true>(W1, W1, ne, prm.dtr, tid, nt);
                __syncthreads();
                // along k in registers: the transposed derivative of the
                // third flux, plus the other two terms, back to the nodes;
                // (Q,Q,P) into W0 (each line reads its own W0 values first)
                kline_pass<Eng, WB, Q, Q>(W3, ne, tid, nt, [&](int, int, int, const V (&x)[Q], const BoxLine<WB, 2>& la) {
                    V t[Q], sv[Q], z[P];
                    eor_line<Eng, Q, Q, -1, true>(x, t, prm.dtr);   // summed next: loose pairs
                    sum_line(t, sv, la);
                    eor_line<Eng, Q, P, +1>(sv, z, prm.bb);
                    line_store<WB, P>(W0, la, z);
                });
            }
            __syncthreads();
            sweep_eor<Eng, WB, 1, Q, Q, P, P, +1>(W0, W1, ne, prm.bb, tid, nt);   // (Q,P,P)
            __syncthreads();
            if constexpr (kDirectIO) {
                interp0_to_dense<Eng, WB, P, Q>(W1, v + e0 * P3, ne, prm.bb, tid, nt);  // -> v
            } else {
                sweep_eor<Eng, WB, 0, Q, P, P, P, +1, true>(W1, W0, ne, prm.bb, tid, nt);   // (P,P,P), stored next
                __syncthreads();
                store_box<Eng, WB, P, P, P>(W0, v + e0 * P3, P3, ne, tid, nt);
            }
            __syncthreads();
        } else {
            load_box<Eng, WB, P, P, P>(us, P3, W0, ne, tid, nt);
            __syncthreads();
            sweep<Eng, WB, 0, P, P, P, Q>(W0, W1, ne, Bi, tid, nt);   // (Q,P,P)
            __syncthreads();
            sweep<Eng, WB, 1, Q, P, P, Q>(W1, W0, ne, Bi, tid, nt);   // (Q,Q,P)
            __syncthreads();
            sweep<Eng, WB, 2, Q, Q, P, Q>(W0, W2, ne, Bi, tid, nt);   // u at the points: W2
            __syncthreads();
            sweep<Eng, WB, 0, Q, Q, Q, Q>(W2, W0, ne, Dg, tid, nt);   // qr
            sweep<Eng, WB, 1, Q, Q, Q, Q>(W2, W1, ne, Dg, tid, nt);   // qs
            sweep<Eng, WB, 2, Q, Q, Q, Q>(W2, W3, ne, Dg, tid, nt);   // qt
            __syncthreads();
            if (ks != nullptr)
                fluxes(std::true_type{});
            else
                fluxes(std::false_type{});
            __syncthreads();
            if (bt + gridDim.x < nbatch) issue(bt + gridDim.x);   // the stage is free
            sweep<Eng, WB, 0, Q, Q, Q, Q>(W0, W0, ne, Dtr, tid, nt);
            sweep<Eng, WB, 1, Q, Q, Q, Q>(W1, W1, ne, Dtr, tid, nt);
            __syncthreads();
            // along r on W3 plus the two other terms -> W2
            kline_pass<Eng, WB, Q, Q>(W3, ne, tid, nt, [&](int, int, int, const V (&x)[Q], const BoxLine<WB, 2>& la) {
                V t[Q], sv[Q];
#pragma unroll
                for (int o = 0; o < Q; ++o) {
                    A acc = Eng::first(Dtr(o, 0), x[0]);
#pragma unroll
                    for (int n = 1; n < Q; ++n) Eng::madd(acc, Dtr(o, n), x[n]);
                    t[o] = Eng::result(acc);
                }
                sum_line(t, sv, la);
                line_store<WB, Q>(W2, la, sv);
            });
            __syncthreads();
            sweep<Eng, WB, 2, Q, Q, Q, P>(W2, W0, ne, Bb, tid, nt);   // (Q,Q,P)
            __syncthreads();
            sweep<Eng, WB, 1, Q, Q, P, P>(W0, W1, ne, Bb, tid, nt);   // (Q,P,P)
            __syncthreads();
            sweep<Eng, WB, 0, Q, P, P, P>(W1, W0, ne, Bb, tid, nt);   // (P,P,P)
            __syncthreads();
            // padded box -> v (consecutive threads, consecutive values)
            store_box<Eng, WB, P, P, P>(W0, v + e0 * P3, P3, ne, tid, nt);
            __syncthreads();
        }
    }
}

}  // namespace bkg
