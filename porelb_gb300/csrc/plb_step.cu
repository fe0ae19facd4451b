/*
 * plb_step.cu - the fused pull-stream + BGK collide + body-force step.
 *
 * One thread per fluid node.  Thread i gathers its 19 post-stream values
 * through the neighbour words (the on-device image of the reference's push
 * stream, stream_inner_nodes porelb.c:285-300), relaxes them (collision,
 * porelb.c:318-365) and writes its 19 post-collision values to the other
 * ping-pong buffer.  Distributions are SoA, f[j][npad], so the 19 stores and
 * the 18 neighbour-word loads of a warp are fully coalesced; the gathers hit
 * nodes that the Morton order keeps close in memory.  In the FP64 form each
 * CTA also asks L2 for the node range of the block half a wave of resident
 * blocks ahead (prefetch_block).
 *
 * Forms:
 *   FP64_EXACT  the reference's operations in the reference's order with
 *               round-to-nearest intrinsics (no FMA contraction): bit-exact.
 *   FP64        exact Q60 fixed-point collision on the integer pipes
 *               (plb_fx.h); nodes outside its range fall back to FP64_FMA.
 *   FP64_FMA    the same algebra in native FP64, restructured for FMA.
 *   FP32/FP16DEV/BF16DEV  relative deviations g = f/w - 1 stored (scaled)
 *               in 32/16/16 bits, collision in FP32 on the deviations.
 */
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include "plb_emu.h"
#include "plb_internal.h"

namespace plb {

/* weights of the three classes, as the reference's doubles (porelb.h:36-42) */
__device__ __forceinline__ double w64(int c)
{
    return c == 0 ? 1.0 / 3 : (c == 1 ? 1.0 / 18 : 1.0 / 36);
}
__device__ __forceinline__ float w32(int c)
{
    return c == 0 ? (float)(1.0 / 3) : (c == 1 ? (float)(1.0 / 18) : (float)(1.0 / 36));
}

__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double dsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }
/* the same product on the integer pipes (plb_emu.h): the same bits for a
 * node whose values, density and run constants passed the range check.
 * The bit-exact collision sends 84 of its 97 products per node here, which
 * balances the FP64 and integer pipes (2.05 -> 2.68 GLUPS at 256^3); a
 * node outside the range takes the NATIVE products. */
template <bool NATIVE>
__device__ __forceinline__ double imul(double a, double b)
{
    if constexpr (NATIVE) {
        return __dmul_rn(a, b);
    } else {
        return __longlong_as_double((long long)emu::dmul_bits_fast(
            (uint64_t)__double_as_longlong(a), (uint64_t)__double_as_longlong(b)));
    }
}

/* ------------------------------------------------------------- gather */

template <typename T>
__device__ __forceinline__ T ldg_t(const T *p) { return __ldg(p); }

template <typename T>
__device__ __forceinline__ void gather(const T *fin, const uint32_t *nbr,
                                       long long np, long long i, T (&f)[Q])
{
    f[0] = ldg_t(fin + i);
#pragma unroll
    for (int j = 1; j < Q; j++) {
        const int w = (int)__ldg(nbr + (long long)(j - 1) * np + i);
        f[j] = ldg_t(fin + ((long long)j * np + w));
    }
}

/* ------------------------------------------------- FP64, reference order */

/* e.u as the reference evaluates ((e0*u + e1*v) + e2*w) (porelb.c:9): terms
 * with a zero coefficient add a signed zero, which changes no result. */
template <int J>
__device__ __forceinline__ double eu_ref(double u, double v, double w)
{
    double acc = 0.0;
    bool first = true;
    if (ex(J) != 0) { acc = ex(J) > 0 ? u : -u; first = false; }
    if (ey(J) != 0) {
        const double t = ey(J) > 0 ? v : -v;
        acc = first ? t : dadd(acc, t);
        first = false;
    }
    if (ez(J) != 0) {
        const double t = ez(J) > 0 ? w : -w;
        acc = first ? t : dadd(acc, t);
        first = false;
    }
    return acc;
}

/* rho_u etc. accumulated in j order (porelb.c:330-336).  The first nonzero
 * term is added to 0.0, which is exact. */
template <int C>
__device__ __forceinline__ double moment_ref(const double (&f)[Q])
{
    double acc = 0.0;
    bool first = true;
#pragma unroll
    for (int j = 0; j < Q; j++) {
        const int e = C == 0 ? ex(j) : (C == 1 ? ey(j) : ez(j));
        if (e == 0) continue;
        if (first) {
            acc = e > 0 ? f[j] : -f[j];
            first = false;
        } else {
            acc = e > 0 ? dadd(acc, f[j]) : dsub(acc, f[j]);
        }
    }
    return acc;
}

struct Macro {
    double rho, u, v, w;
    bool bad;
};

template <bool NATIVE>
__device__ __forceinline__ Macro collide_fp64_exact(double (&f)[Q],
                                                     const Coeffs &a, uint32_t &outside)
{
    Macro m;
    double rho = f[0];
#pragma unroll
    for (int j = 1; j < Q; j++) rho = dadd(rho, f[j]);
    double ru = moment_ref<0>(f);
    const double rv = moment_ref<1>(f);
    const double rw = moment_ref<2>(f);
    m.bad = (rho > 1.2) | (rho < 0.5);
    if constexpr (!NATIVE) {
        /* the density in [2^-64, 2^64) too, or the node takes the native
         * multiply (the caller) */
        const uint64_t rb = (uint64_t)__double_as_longlong(rho);
        outside |= emu::outside_node_range(rb) | (uint32_t)((rb << 1) == 0ull);
        if (outside) return m;
    }
    if (a.it > 0) ru = dadd(ru, a.half_force);
    const double u = __ddiv_rn(ru, rho);
    const double v = __ddiv_rn(rv, rho);
    const double w = __ddiv_rn(rw, rho);
    m.rho = rho; m.u = u; m.v = v; m.w = w;

    const double uv = dadd(dadd(dmul(u, u), dmul(v, v)), dmul(w, w));
    const double uv15 = dmul(1.5, uv);
    const double h0 = dmul(w64(0), rho);
    const double h1 = dmul(w64(1), rho);
    const double h2 = dmul(w64(2), rho);
    /* omega + ((1-omega/2)*3*(e_x - u))*F for e_x = -1, 0, +1 */
    const double am = dadd(a.omega, dmul(dmul(a.k3, dsub(-1.0, u)), a.force));
    const double a0 = dadd(a.omega, dmul(dmul(a.k3, dsub(0.0, u)), a.force));
    const double ap = dadd(a.omega, dmul(dmul(a.k3, dsub(1.0, u)), a.force));

    /* rest direction: e.u = 0 gives ((1 + 0) + 0) - 1.5 uv */
    {
        const double feq = imul<NATIVE>(h0, dsub(1.0, uv15));
        f[0] = dadd(imul<NATIVE>(a.om1, f[0]), imul<NATIVE>(a0, feq));
    }
    /* pairs (J, J+1) with e_{J+1} = -e_J: 3 e.u, 4.5 e.u and (4.5 e.u) e.u
     * of the partner are exact negations / the same value. */
#pragma unroll
    for (int J = 1; J < Q; J += 2) {
        const int K = J + 1;
        const double eu = (J == 1) ? eu_ref<1>(u, v, w)
                        : (J == 3) ? eu_ref<3>(u, v, w)
                        : (J == 5) ? eu_ref<5>(u, v, w)
                        : (J == 7) ? eu_ref<7>(u, v, w)
                        : (J == 9) ? eu_ref<9>(u, v, w)
                        : (J == 11) ? eu_ref<11>(u, v, w)
                        : (J == 13) ? eu_ref<13>(u, v, w)
                        : (J == 15) ? eu_ref<15>(u, v, w)
                                    : eu_ref<17>(u, v, w);
        const double t3 = imul<NATIVE>(3.0, eu);
        const double c2 = imul<NATIVE>(imul<NATIVE>(4.5, eu), eu);
        const double h = wclass(J) == 1 ? h1 : h2;
        const double feqJ = imul<NATIVE>(h, dsub(dadd(dadd(1.0, t3), c2), uv15));
        const double feqK = imul<NATIVE>(h, dsub(dadd(dsub(1.0, t3), c2), uv15));
        const double AJ = ex(J) > 0 ? ap : (ex(J) < 0 ? am : a0);
        const double AK = ex(K) > 0 ? ap : (ex(K) < 0 ? am : a0);
        f[J] = dadd(imul<NATIVE>(a.om1, f[J]), imul<NATIVE>(AJ, feqJ));
        f[K] = dadd(imul<NATIVE>(a.om1, f[K]), imul<NATIVE>(AK, feqK));
    }
    return m;
}

/* ------------------------------------------------------ FP64 with FMA */

__device__ __forceinline__ Macro collide_fp64_fma(double (&f)[Q],
                                                   const Coeffs &a)
{
    Macro m;
    double s[Q], d[Q];
#pragma unroll
    for (int J = 1; J < Q; J += 2) {
        s[J] = f[J] + f[J + 1];
        d[J] = f[J] - f[J + 1];
    }
    double rho = f[0];
#pragma unroll
    for (int J = 1; J < Q; J += 2) rho += s[J];
    double jx = 0.0, jy = 0.0, jz = 0.0;
#pragma unroll
    for (int J = 1; J < Q; J += 2) {
        if (ex(J)) jx += ex(J) * d[J];
        if (ey(J)) jy += ey(J) * d[J];
        if (ez(J)) jz += ez(J) * d[J];
    }
    m.bad = (rho > 1.2) | (rho < 0.5);
    if (a.it > 0) jx += a.half_force;
    const double inv = 1.0 / rho;
    const double u = jx * inv, v = jy * inv, w = jz * inv;
    m.rho = rho; m.u = u; m.v = v; m.w = w;
    const double uv15 = 1.5 * (u * u + v * v + w * w);
    const double c = a.k3 * a.force;
    const double am = a.omega - c * (1.0 + u);
    const double a0 = a.omega - c * u;
    const double ap = a.omega + c * (1.0 - u);
    const double h0 = w64(0) * rho, h1 = w64(1) * rho, h2 = w64(2) * rho;
    const double b1 = h1 - h1 * uv15, b2 = h2 - h2 * uv15;
    f[0] = a.om1 * f[0] + a0 * (h0 - h0 * uv15);
#pragma unroll
    for (int J = 1; J < Q; J += 2) {
        const int K = J + 1;
        const double eu = ex(J) * u + ey(J) * v + ez(J) * w;
        const double h = wclass(J) == 1 ? h1 : h2;
        const double b = wclass(J) == 1 ? b1 : b2;
        const double sym = fma(4.5 * h * eu, eu, b);
        const double anti = 3.0 * h * eu;
        const double AJ = ex(J) > 0 ? ap : (ex(J) < 0 ? am : a0);
        const double AK = ex(K) > 0 ? ap : (ex(K) < 0 ? am : a0);
        f[J] = fma(a.om1, f[J], AJ * (sym + anti));
        f[K] = fma(a.om1, f[K], AK * (sym - anti));
    }
    return m;
}

/* ----------------------------------------- FP32 collision on deviations */

/* g_j = f_j / w_j - 1.  With rho = 1 + delta, the BGK + force update
 *   f' = (1-omega) f + (omega + a_j) w rho (1 + P_j),
 *   a_j = 3 (1 - omega/2) F (e_jx - u),  P_j = 3 e.u + 4.5 (e.u)^2 - 1.5 u.u
 * becomes, exactly in real arithmetic,
 *   g'_j = (1-omega) g_j + omega delta + rho ((omega + a_j) P_j + a_j),
 * which keeps every FP32 quantity at deviation scale. */
__device__ __forceinline__ Macro collide_dev32(float (&g)[Q], const Coeffs &a)
{
    Macro m;
    float d[Q];
#pragma unroll
    for (int j = 0; j < Q; j++) d[j] = w32(wclass(j)) * g[j];
    float s[Q], df[Q];
#pragma unroll
    for (int J = 1; J < Q; J += 2) {
        s[J] = d[J] + d[J + 1];
        df[J] = d[J] - d[J + 1];
    }
    float delta = d[0];
#pragma unroll
    for (int J = 1; J < Q; J += 2) delta += s[J];
    float jx = 0.f, jy = 0.f, jz = 0.f;
#pragma unroll
    for (int J = 1; J < Q; J += 2) {
        if (ex(J)) jx += ex(J) * df[J];
        if (ey(J)) jy += ey(J) * df[J];
        if (ez(J)) jz += ez(J) * df[J];
    }
    const float rho = 1.0f + delta;
    m.bad = (rho > 1.2f) | (rho < 0.5f);
    if (a.it > 0) jx += a.half_force_f;
    const float inv = 1.0f / rho;
    const float u = jx * inv, v = jy * inv, w = jz * inv;
    m.rho = 1.0 + (double)delta;
    m.u = u; m.v = v; m.w = w;
    const float om = a.omega_f, om1 = a.om1_f;
    const float c = a.c_f;
    const float uv15 = 1.5f * (u * u + v * v + w * w);
    const float base = om * delta;
    const float am = -c * (1.0f + u), a0 = -c * u, ap = c * (1.0f - u);
    {
        const float P = -uv15;
        g[0] = fmaf(om1, g[0], base + rho * fmaf(om + a0, P, a0));
    }
#pragma unroll
    for (int J = 1; J < Q; J += 2) {
        const int K = J + 1;
        const float eu = ex(J) * u + ey(J) * v + ez(J) * w;
        const float sym = fmaf(4.5f * eu, eu, -uv15);
        const float PJ = fmaf(3.0f, eu, sym);
        const float PK = fmaf(-3.0f, eu, sym);
        const float aJ = ex(J) > 0 ? ap : (ex(J) < 0 ? am : a0);
        const float aK = ex(K) > 0 ? ap : (ex(K) < 0 ? am : a0);
        g[J] = fmaf(om1, g[J], base + rho * fmaf(om + aJ, PJ, aJ));
        g[K] = fmaf(om1, g[K], base + rho * fmaf(om + aK, PK, aK));
    }
    return m;
}

/* storage conversion of the deviation forms */
__device__ __forceinline__ float to_f(float x) { return x; }
__device__ __forceinline__ float to_f(__half x) { return __half2float(x); }
__device__ __forceinline__ float to_f(__nv_bfloat16 x) { return __bfloat162float(x); }
template <typename T> __device__ __forceinline__ T from_f(float x);
template <> __device__ __forceinline__ float from_f<float>(float x) { return x; }
template <> __device__ __forceinline__ __half from_f<__half>(float x) { return __float2half_rn(x); }
template <> __device__ __forceinline__ __nv_bfloat16 from_f<__nv_bfloat16>(float x) { return __float2bfloat16_rn(x); }

/* --------------------------------------------------------------- kernel */

/* ----------------------------------------- FP64 on the integer pipes */

template <bool MACRO>
__device__ __forceinline__ Macro collide_fx(double (&f)[Q], const Coeffs &a,
                                            bool &fallback)
{
    uint64_t b[Q];
#pragma unroll
    for (int j = 0; j < Q; j++) b[j] = (uint64_t)__double_as_longlong(f[j]);
    fx::Moments mm;
    const uint32_t fl = fx::collide(b, a.fxk, a.it > 0, mm);
    Macro m;
    fallback = (fl & fx::kBad) != 0;
    m.bad = (fl & fx::kDensity) != 0;
#pragma unroll
    for (int j = 0; j < Q; j++) f[j] = __longlong_as_double((long long)b[j]);
    if (MACRO) {
        uint32_t ignore = 0;
        m.rho = __longlong_as_double((long long)fx::to_bits(mm.R, ignore));
        m.u = (double)fx::mul(mm.Jx, mm.inv) * 0x1p-60;
        m.v = (double)fx::mul(mm.Jy, mm.inv) * 0x1p-60;
        m.w = (double)fx::mul(mm.Jz, mm.inv) * 0x1p-60;
    } else {
        m.rho = m.u = m.v = m.w = 0.0;
    }
    return m;
}

template <int PREC> struct StoreOf { using T = double; };
template <> struct StoreOf<PLB_FP32> { using T = float; };
template <> struct StoreOf<PLB_FP16DEV> { using T = __half; };
template <> struct StoreOf<PLB_BF16DEV> { using T = __nv_bfloat16; };

/* Resident blocks of 256 threads per SM the register budget is set for,
 * by kernel variant (0 = default; 1 and 3 the alternatives the launch tuner
 * tries): fixed-point FP64 128 / 80 / 64 registers, the FP32 and 16-bit
 * forms 48 / unconstrained / 40 registers (48 is the faster on GB300: FP16
 * deviations 39.1 against 38.4 GLUPS at 512^3), the other FP64 forms
 * unconstrained. */
template <int PREC, int V> struct MinBlocks {
    static constexpr bool dev = PREC == PLB_FP32 || PREC == PLB_FP16DEV || PREC == PLB_BF16DEV;
    static constexpr int v = PREC == PLB_FP64 ? (V == 1 ? 3 : V == 3 ? 4 : 2)
                           : dev ? (V == 1 ? 1 : V == 3 ? 6 : 5)
                                 : 1;
};

/* Gather, collide and store node i.  Returns the macros; *dev_max receives
 * the largest stored deviation magnitude of the 16-bit forms. */
/* The bit-exact collision of node i with every product on the FP64 pipe,
 * from its streamed values gathered again, stored: the path of a node
 * whose values or density (or the run's constants) lie outside the range
 * of the integer multiply's check, such as an infinity, a NaN, a subnormal
 * or an extreme value.  Out of line, so the common path keeps its
 * registers. */
__device__ __noinline__ Macro exact_node_native(const double *fin, double *fout,
                                                const uint32_t *nbr, long long np,
                                                long long i, const Coeffs &co)
{
    double raw[Q];
    gather<double>(fin, nbr, np, i, raw);
    uint32_t unused = 0;
    const Macro m = collide_fp64_exact<true>(raw, co, unused);
#pragma unroll
    for (int j = 0; j < Q; j++) __stcs(fout + (long long)j * np + i, raw[j]);
    return m;
}

/* Collide node i's streamed values raw[] and store them. */
template <int PREC, bool MACRO, typename T>
__device__ __forceinline__ Macro collide_node(T (&raw)[Q], const T *fin, T *fout,
                                              const uint32_t *nbr, long long np,
                                              long long i, const Coeffs &co,
                                              unsigned int &flags, float &dev_max)
{
    Macro m;
    if constexpr (PREC == PLB_FP64) {
        bool fallback;
        m = collide_fx<MACRO>(raw, co, fallback);
        if (fallback) {
            /* outside the fixed-point range: native FP64 from the streamed
             * values, gathered again */
            gather<T>(fin, nbr, np, i, raw);
            m = collide_fp64_fma(raw, co);
            flags |= 2u;
        }
#pragma unroll
        for (int j = 0; j < Q; j++) __stcs(fout + (long long)j * np + i, raw[j]);
    } else if constexpr (PREC == PLB_FP64_EXACT || PREC == PLB_FP64_FMA) {
        if constexpr (PREC == PLB_FP64_EXACT) {
            /* the integer multiply needs the node's values in [2^-64, 2^64)
             * (and its density, checked in the collision): their smallest
             * and largest exponent field (a zero value, which the range
             * admits but a distribution never is, takes the native path) */
            uint32_t emin = 0x7ffu, emax = 0u;
#pragma unroll
            for (int j = 0; j < Q; j++) {
                const uint32_t e = ((uint32_t)__double2hiint(raw[j]) >> 20) & 0x7ffu;
                emin = min(emin, e);
                emax = max(emax, e);
            }
            uint32_t outside = (uint32_t)co.exact_native | (uint32_t)(emin < 1023u - 64u) |
                               (uint32_t)(emax > 1023u + 63u);
            if (!outside) m = collide_fp64_exact<false>(raw, co, outside);
            if (outside) {
                flags |= 2u;
                return exact_node_native(fin, fout, nbr, np, i, co);
            }
        } else {
            m = collide_fp64_fma(raw, co);
        }
#pragma unroll
        for (int j = 0; j < Q; j++) __stcs(fout + (long long)j * np + i, raw[j]);
    } else {
        float g[Q];
#pragma unroll
        for (int j = 0; j < Q; j++) g[j] = to_f(raw[j]) * co.inv_scale;
        m = collide_dev32(g, co);
        float big = 0.f;
#pragma unroll
        for (int j = 0; j < Q; j++) {
            const float h = g[j] * co.scale;
            big = fmaxf(big, fabsf(h));
            fout[(long long)j * np + i] = from_f<T>(h);
        }
        if (PREC == PLB_FP16DEV && !(big <= 60000.f)) flags |= 1u;
        dev_max = big;
    }
    return m;
}

/* Gather, collide and store node i.  Returns the macros; dev_max receives
 * the largest stored deviation magnitude of the 16-bit forms. */
template <int PREC, bool MACRO>
__device__ __forceinline__ Macro step_node(const void *fin_, void *fout_,
                                           const uint32_t *nbr, long long np,
                                           long long i, const Coeffs &co,
                                           unsigned int &flags, float &dev_max)
{
    using T = typename StoreOf<PREC>::T;
    const T *fin = (const T *)fin_;
    T raw[Q];
    gather<T>(fin, nbr, np, i, raw);
    return collide_node<PREC, MACRO>(raw, fin, (T *)fout_, nbr, np, i, co, flags, dev_max);
}

/* Bulk L2 prefetch of [p, p + bytes), bytes a positive multiple of 16 and
 * p 16-byte aligned. */
__device__ __forceinline__ void prefetch_l2(const void *p, unsigned bytes)
{
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(p), "r"(bytes) : "memory");
}

/* Thread 0 of a block asks L2 for the node range of block b (a block that
 * starts some time after this one, pf_blocks blocks later in launch order):
 * its 18 rows of neighbour words and its 19 rows of distributions.  In
 * Morton order most gathers of that block read inside the ranges of the
 * blocks launched near it, so its loads then wait for L2 instead of DRAM.  Rows are npad elements (a
 * multiple of 64) and the block size is a multiple of 32, so every range
 * starts 64-byte aligned and spans a multiple of 64 bytes inside its row. */
template <typename T>
__device__ __forceinline__ void prefetch_block(const T *fin, const uint32_t *nbr,
                                               long long np, long long n, long long b,
                                               int bs)
{
    const long long i0 = b * bs;
    if (i0 >= n) return;
    const long long cnt = np - i0 < bs ? np - i0 : bs;
    const unsigned wb = (unsigned)(cnt * 4);
    const unsigned fb = (unsigned)(cnt * (long long)sizeof(T));
#pragma unroll 1
    for (int j = 0; j < Q - 1; j++) prefetch_l2(nbr + (long long)j * np + i0, wb);
#pragma unroll 1
    for (int j = 0; j < Q; j++) prefetch_l2(fin + (long long)j * np + i0, fb);
}

template <int PREC, bool MACRO, int VARIANT>
__global__ void __launch_bounds__(256, MinBlocks<PREC, VARIANT>::v)
k_step(const StepArgs a)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (a.pf_blocks > 0 && threadIdx.x == 0)
        prefetch_block<typename StoreOf<PREC>::T>((const typename StoreOf<PREC>::T *)a.fin,
                                                  a.nbr, a.npad, a.n,
                                                  (long long)blockIdx.x + a.pf_blocks,
                                                  blockDim.x);
    double sum_u = 0.0, sum_r = 0.0;
    if (i < a.n) {
        float dm = 0.f;
        unsigned int fl = 0;
        const Macro m = step_node<PREC, MACRO>(a.fin, a.fout, a.nbr, a.npad, i, a.co,
                                               fl, dm);
        if (fl) atomicOr(a.flags, fl);
        if (m.bad) {
            const unsigned long long key =
                ((unsigned long long)(unsigned)a.co.it << 32) | (unsigned)a.perm[i];
            atomicMin(a.err, key);
        }
        if (MACRO) {
            const long long np = a.npad;
            a.macro[i] = m.rho;
            a.macro[np + i] = m.u;
            a.macro[2 * np + i] = m.v;
            a.macro[3 * np + i] = m.w;
            sum_u = m.u;
            sum_r = m.rho;
        }
    }
    if (MACRO) {
        __shared__ double su[32], sr[32];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            sum_u += __shfl_down_sync(0xffffffffu, sum_u, o);
            sum_r += __shfl_down_sync(0xffffffffu, sum_r, o);
        }
        const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
        if (lane == 0) { su[wid] = sum_u; sr[wid] = sum_r; }
        __syncthreads();
        if (threadIdx.x == 0) {
            double tu = 0.0, tr = 0.0;
            for (int k = 0; k < (int)(blockDim.x >> 5); k++) { tu += su[k]; tr += sr[k]; }
            a.partial[blockIdx.x] = tu;
            a.partial[gridDim.x + blockIdx.x] = tr;
        }
    }
}

/* Batch step: kBatchBlock / BT CTAs of BT threads per active pool block;
 * CTA b works on part b % H of pool block blk_list[b / H] (of the current
 * L2 group's window of the list, when the pool steps in groups), whose map
 * entry blk_sample[] packs its sample and that sample's node count in it.  CTAs
 * that run at the same time work on neighbouring pool blocks, so in Morton
 * order their gathers share L2 lines (a fixed grid looping over the list
 * lost that and ran 23% slower in the FP64 form). */
template <int PREC, bool MACRO, int BT>
__global__ void __launch_bounds__(BT, MinBlocks<PREC, 0>::v * (kBatchBlock / BT))
k_batch_step(const BatchArgs a)
{
    using T = typename StoreOf<PREC>::T;
    constexpr int H = kBatchBlock / BT; /* CTAs per pool block */
    const int *list = a.blk_list;
    int ncta = (int)gridDim.x;
    if (a.grp) {
        /* one L2 group of the interval: its window of the block list */
        const int g = *a.grp_cur;
        list += a.grp[2 * g];
        ncta = a.grp[2 * g + 1] * H;
        if ((int)blockIdx.x >= ncta) return;
    }
    const int part = blockIdx.x % H;
    const int pb = list[blockIdx.x / H];
    const int packed = a.blk_sample[pb];
    const int s = packed >> 9;                  /* -1: free block */
    const int k = part * BT + threadIdx.x;      /* node within the pool block */
    const bool valid = s >= 0 && k < (packed & 511);
    const long long i = (long long)pb * kBatchBlock + k;
    /* L2 prefetch of the part of a pool block the CTA pf_blocks later steps */
    if (a.pf_blocks > 0 && threadIdx.x == 0 && (int)blockIdx.x + a.pf_blocks < ncta) {
        const unsigned c = blockIdx.x + a.pf_blocks;
        prefetch_block<T>((const T *)a.fin, a.nbr, a.npad, a.npad,
                          (long long)list[c / H] * H + c % H, BT);
    }
    double sum_u = 0.0, sum_r = 0.0;
    float dmax = 0.f;
    /* the gathers first: they need only the node's place in the pool */
    T raw[Q];
    if (valid) gather<T>((const T *)a.fin, a.nbr, a.npad, i, raw);
    if (valid) {
        {
            /* the sample's coefficients straight from global memory (the
             * same record for the whole CTA: cached after the first warp);
             * no shared-memory staging, so no barrier makes the warps wait
             * for each other's gathers */
            const SampleDev *sp = a.samples + s;
            Coeffs co = sp->co;
            co.it = *a.t_base + a.t_off - sp->start;
            unsigned int fl = 0;
            const Macro m = collide_node<PREC, MACRO>(raw, (const T *)a.fin, (T *)a.fout,
                                                      a.nbr, a.npad, i, co, fl, dmax);
            if (fl | (m.bad ? 4u : 0u)) atomicOr(a.serr + s, fl | (m.bad ? 4u : 0u));
            if (MACRO) {
                const long long np = a.npad;
                if (a.macro) {
                    a.macro[i] = m.rho;
                    a.macro[np + i] = m.u;
                    a.macro[2 * np + i] = m.v;
                    a.macro[3 * np + i] = m.w;
                }
                sum_u = m.u;
                sum_r = m.rho;
            }
        }
    }
    if (MACRO) {
        __shared__ double su[32], sr[32];
        __shared__ float sd[32];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            sum_u += __shfl_down_sync(0xffffffffu, sum_u, o);
            sum_r += __shfl_down_sync(0xffffffffu, sum_r, o);
            dmax = fmaxf(dmax, __shfl_down_sync(0xffffffffu, dmax, o));
        }
        const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
        if (lane == 0) { su[wid] = sum_u; sr[wid] = sum_r; sd[wid] = dmax; }
        __syncthreads();
        if (threadIdx.x == 0) {
            double tu = 0.0, tr = 0.0;
            float td = 0.f;
            for (int w = 0; w < BT / 32; w++) {
                tu += su[w];
                tr += sr[w];
                td = fmaxf(td, sd[w]);
            }
            const long long row = (long long)pb * H + part;
            a.partial[row] = tu;
            a.partial[a.part_stride + row] = tr;
            a.partial[2 * a.part_stride + row] = (double)td;
        }
    }
}

template <int PREC>
static cudaError_t launch_prec(bool macros, const StepArgs &a, int block,
                               int variant, cudaStream_t s)
{
    const int grid = (a.n + block - 1) / block;
    if (grid == 0) return cudaSuccess;
    /* the tighter budgets are built for the tuned forms only */
    constexpr bool tuned = PREC == PLB_FP64 || PREC == PLB_FP32 || PREC == PLB_FP16DEV ||
                           PREC == PLB_BF16DEV;
    if constexpr (tuned) {
        if (variant == 1) {
            if (macros) k_step<PREC, true, 1><<<grid, block, 0, s>>>(a);
            else k_step<PREC, false, 1><<<grid, block, 0, s>>>(a);
            return cudaGetLastError();
        }
        if (variant == 3) {
            if (macros) k_step<PREC, true, 3><<<grid, block, 0, s>>>(a);
            else k_step<PREC, false, 3><<<grid, block, 0, s>>>(a);
            return cudaGetLastError();
        }
    }
    if (macros) k_step<PREC, true, 0><<<grid, block, 0, s>>>(a);
    else k_step<PREC, false, 0><<<grid, block, 0, s>>>(a);
    return cudaGetLastError();
}

/* Blocks of the (non-macro) step kernel resident on the whole device at
 * once: the L2 prefetch distance. */
template <int PREC>
static int wave_prec(int block, int variant)
{
    const void *fn = (const void *)k_step<PREC, false, 0>;
    constexpr bool tuned = PREC == PLB_FP64 || PREC == PLB_FP32 || PREC == PLB_FP16DEV ||
                           PREC == PLB_BF16DEV;
    if constexpr (tuned) {
        if (variant == 1) fn = (const void *)k_step<PREC, false, 1>;
        if (variant == 3) fn = (const void *)k_step<PREC, false, 3>;
    }
    int dev = 0, sms = 0, per = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, fn, block, 0) != cudaSuccess)
        return 0;
    return sms * per;
}

int step_wave_blocks(int precision, int block, int variant)
{
    switch (precision) {
    case PLB_FP64_EXACT: return wave_prec<PLB_FP64_EXACT>(block, variant);
    case PLB_FP64: return wave_prec<PLB_FP64>(block, variant);
    case PLB_FP64_FMA: return wave_prec<PLB_FP64_FMA>(block, variant);
    case PLB_FP32: return wave_prec<PLB_FP32>(block, variant);
    case PLB_FP16DEV: return wave_prec<PLB_FP16DEV>(block, variant);
    case PLB_BF16DEV: return wave_prec<PLB_BF16DEV>(block, variant);
    default: return 0;
    }
}

/* Threads per CTA of the batch step by default: 128 for the fixed-point
 * FP64 form (two CTAs per pool block; 4% faster in the plain kernel), 256
 * otherwise.  A pool may choose either (the launch tuner times both). */
int batch_default_cta(int precision)
{
    return precision == PLB_FP64 ? 128 : kBatchBlock;
}

template <int PREC, int BT>
static int batch_wave_bt()
{
    int dev = 0, sms = 0, per = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_batch_step<PREC, false, BT>, BT,
                                                      0) != cudaSuccess)
        return 0;
    return sms * per;
}

template <int PREC>
static int batch_wave_prec(int cta)
{
    return cta == 128 ? batch_wave_bt<PREC, 128>() : batch_wave_bt<PREC, kBatchBlock>();
}

int batch_wave_blocks(int precision, int cta)
{
    switch (precision) {
    case PLB_FP64_EXACT: return batch_wave_prec<PLB_FP64_EXACT>(cta);
    case PLB_FP64: return batch_wave_prec<PLB_FP64>(cta);
    case PLB_FP64_FMA: return batch_wave_prec<PLB_FP64_FMA>(cta);
    case PLB_FP32: return batch_wave_prec<PLB_FP32>(cta);
    case PLB_FP16DEV: return batch_wave_prec<PLB_FP16DEV>(cta);
    case PLB_BF16DEV: return batch_wave_prec<PLB_BF16DEV>(cta);
    default: return 0;
    }
}

template <int PREC>
static const void *batch_fn(bool macros, int cta)
{
    if (cta == 128)
        return macros ? (const void *)k_batch_step<PREC, true, 128>
                      : (const void *)k_batch_step<PREC, false, 128>;
    return macros ? (const void *)k_batch_step<PREC, true, kBatchBlock>
                  : (const void *)k_batch_step<PREC, false, kBatchBlock>;
}

const void *batch_step_kernel(int precision, bool macros, int cta)
{
    if (cta != 128 && cta != kBatchBlock) return nullptr;
    switch (precision) {
    case PLB_FP64_EXACT: return batch_fn<PLB_FP64_EXACT>(macros, cta);
    case PLB_FP64: return batch_fn<PLB_FP64>(macros, cta);
    case PLB_FP64_FMA: return batch_fn<PLB_FP64_FMA>(macros, cta);
    case PLB_FP32: return batch_fn<PLB_FP32>(macros, cta);
    case PLB_FP16DEV: return batch_fn<PLB_FP16DEV>(macros, cta);
    case PLB_BF16DEV: return batch_fn<PLB_BF16DEV>(macros, cta);
    default: return nullptr;
    }
}

cudaError_t launch_step(int precision, bool macros, const StepArgs &a,
                        int block, int variant, cudaStream_t s)
{
    switch (precision) {
    case PLB_FP64_EXACT: return launch_prec<PLB_FP64_EXACT>(macros, a, block, variant, s);
    case PLB_FP64: return launch_prec<PLB_FP64>(macros, a, block, variant, s);
    case PLB_FP64_FMA: return launch_prec<PLB_FP64_FMA>(macros, a, block, variant, s);
    case PLB_FP32: return launch_prec<PLB_FP32>(macros, a, block, variant, s);
    case PLB_FP16DEV: return launch_prec<PLB_FP16DEV>(macros, a, block, variant, s);
    case PLB_BF16DEV: return launch_prec<PLB_BF16DEV>(macros, a, block, variant, s);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace plb
