/*
 * md_pair.cuh -- the per-pair force law shared by the pair kernels.
 *
 * pair_forces.cu:34-205: for each listed j inside rc,
 *   Wolf:  ff = qfac qi qj ([2a/sqrt(pi) r + P5(t) t] e^{-a^2 r^2} / r - W) / r^2,
 *          t = 1/(1 + p a r), P5 = A&S 7.1.26 (simulation.h:39-44),
 *   RF:    ff = qfac qi qj (1/r - k_rf r^2) / r^2,
 *   + LJ:  ff += lj1 r^-14 - lj2 r^-8,
 * F_i += ff d, w_i += ff r^2.
 */
#ifndef MD_PAIR_CUH
#define MD_PAIR_CUH

#include "md_device.cuh"

namespace {

#define A1 0.254829592f
#define A2 -0.284496736f
#define A3 1.421413741f
#define A4 -1.453152027f
#define A5 1.061405429f
#define QFAC 1389.35427611722f

struct pair_consts {
    float ucc;     /* Coulomb energy shift at rc */
    float rc6i;    /* rc^-6 */
    float rcinv;   /* 1/rc */
};

/* Round to nearest even for |t| < 2^22 with two FP32 adds (no conversion
 * instruction): the minimum-image shift rint(d / L). */
__device__ __forceinline__ float rint_small(float t)
{
    const float M = 12582912.0f;   /* 1.5 * 2^23 */
    return __fsub_rn(__fadd_rn(t, M), M);
}

/* The hardware approximations (PTX ISA ex2/rsqrt/rcp .approx.ftz): relative
 * errors ~2^-22, well inside the 1e-5 force tolerance; arguments here are
 * never denormal. */
__device__ __forceinline__ float ex2_approx(float x)
{
    float y;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float rsqrt_approx(float x)
{
    float y;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float rcp_approx(float x)
{
    float y;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

struct pair_acc {
    float fx, fy, fz, fw, fe;
};

/* Geometry and force-law constants seen by an atom.  geom_kp reads them
 * from the kernel parameters (a single system); geom_reg holds a copy in
 * registers (one replica of a batch). */
struct geom_kp {
    const md_kparams &kp;
    const pair_consts &pc;
    __device__ __forceinline__ float L(int d) const { return kp.box[d]; }
    __device__ __forceinline__ float Li(int d) const { return kp.boxi[d]; }
    __device__ __forceinline__ float rcsq() const { return kp.rcutsq; }
    __device__ __forceinline__ float reacf() const { return kp.reacf; }
    __device__ __forceinline__ float palfa() const { return kp.palfa; }
    __device__ __forceinline__ float spiialfa() const { return kp.spiialfa; }
    __device__ __forceinline__ float alfasq() const { return kp.alfasq; }
    __device__ __forceinline__ float wolf() const { return kp.wolf; }
    __device__ __forceinline__ float ucc() const { return pc.ucc; }
    __device__ __forceinline__ float rc6i() const { return pc.rc6i; }
    __device__ __forceinline__ float rcinv() const { return pc.rcinv; }
    __device__ __forceinline__ bool centered() const { return kp.centered != 0; }
};

struct geom_reg {
    float L_[3], Li_[3], rcsq_, reacf_, palfa_, spiialfa_, alfasq_, wolf_, ucc_, rc6i_, rcinv_;
    bool centered_;
    __device__ __forceinline__ float L(int d) const { return L_[d]; }
    __device__ __forceinline__ float Li(int d) const { return Li_[d]; }
    __device__ __forceinline__ float rcsq() const { return rcsq_; }
    __device__ __forceinline__ float reacf() const { return reacf_; }
    __device__ __forceinline__ float palfa() const { return palfa_; }
    __device__ __forceinline__ float spiialfa() const { return spiialfa_; }
    __device__ __forceinline__ float alfasq() const { return alfasq_; }
    __device__ __forceinline__ float wolf() const { return wolf_; }
    __device__ __forceinline__ float ucc() const { return ucc_; }
    __device__ __forceinline__ float rc6i() const { return rc6i_; }
    __device__ __forceinline__ float rcinv() const { return rcinv_; }
    __device__ __forceinline__ bool centered() const { return centered_; }
};

/* The register geometry of one replica of a batch; centered: every position
 * of the batch lies inside its replica's box, centred on the origin. */
__device__ __forceinline__ geom_reg rep_geom(const md_rep &R, bool centered = false)
{
    geom_reg g;
    g.centered_ = centered;
    for (int d = 0; d < 3; d++) {
        g.L_[d] = R.box[d];
        g.Li_[d] = R.boxi[d];
    }
    g.rcsq_ = R.rcutsq;
    g.reacf_ = R.reacf;
    g.palfa_ = R.palfa;
    g.spiialfa_ = R.spiialfa;
    g.alfasq_ = R.alfasq;
    g.wolf_ = R.wolf;
    g.ucc_ = R.ucc;
    g.rc6i_ = R.rc6i;
    g.rcinv_ = R.rcinv;
    return g;
}

/* The x and y minimum-image constants of one entry as register pairs:
 * (1/Lx, 1/Ly), (-Lx, -Ly) and 1.5 * 2^23 in both halves. */
struct wrapxy {
    v2<true> li, nl, magic;
    template <class G>
    __device__ __forceinline__ static wrapxy make(const G &g)
    {
        wrapxy w;
        w.li = v2<true>::make(g.Li(0), g.Li(1));
        w.nl = v2<true>::make(-g.L(0), -g.L(1));
        w.magic = v2<true>::make(12582912.0f, 12582912.0f);
        return w;
    }
};

/* One pair: F_i += ff d, w_i += ff r^2 (pair_forces.cu:165-200 / :74-120).
 * x and y of the difference and of its minimum-image shift go through
 * packed f32x2 instructions (PXY = (x_i, y_i); x_j, y_j are the low half of
 * the loaded float4), z through scalar ones; each half rounds as the scalar
 * form (the shift's multiply and add may be contracted, which matters only
 * for |d| = L/2, beyond rc).  WRAP = false skips the minimum-image shift,
 * which is then zero for every pair inside rc (atom i at least rc from each
 * face: see interior()). */
template <int KIND, bool ENERGY, bool WRAP = true, class G>
__device__ __forceinline__ void pair_term(const G &g, const wrapxy &W, v2<true> PXY, float4 pi, float qi,
                                          float4 pj, float2 l, bool valid, pair_acc &a)
{
    typedef v2<true> V;
    V dxy = PXY - V::make(pj.x, pj.y);
    float dz = pi.z - pj.z;
    if (WRAP) {
        dxy = V::fma(W.nl, (dxy * W.li + W.magic) - W.magic, dxy);
        dz -= g.L(2) * rint_small(dz * g.Li(2));
    }
    float dx, dy;
    dxy.get(dx, dy);
    float rsq = dx * dx + dy * dy + dz * dz;
    float ri = rsqrt_approx(rsq);
    float ri2 = ri * ri;
    float qq = qi * pj.w;
    float ff, uc = 0.0f;
    if (KIND == 1) {
        float r = rsq * ri;
        float t = rcp_approx(1.0f + g.palfa() * r);
        float poly = ((((A5 * t + A4) * t + A3) * t + A2) * t + A1) * t;
        float ex = ex2_approx(g.alfasq() * rsq);
        ff = ((g.spiialfa() * r + poly) * ex * ri - g.wolf()) * qq;
        if (ENERGY) uc = qq * (poly * ex * ri - g.ucc() + g.wolf() * __logf(r * g.rcinv()));
    } else {
        ff = qq * (ri - g.reacf() * rsq);
        if (ENERGY) uc = qq * (ri + 0.5f * g.reacf() * rsq - g.ucc());
    }
    float ri6 = ri2 * ri2 * ri2;
    ff = ff * ri2 + (l.x * ri6 - l.y) * ri6 * ri2;
    /* list padding entries point at the atom itself: r = 0 is skipped */
    bool in = valid && rsq <= g.rcsq() && rsq > 0.0f;
    ff = in ? ff : 0.0f;
    a.fx += ff * dx;
    a.fy += ff * dy;
    a.fz += ff * dz;
    a.fw += ff * rsq;
    if (ENERGY) {
        float ulj = l.x * (1.0f / 12.0f) * (ri6 * ri6 - g.rc6i() * g.rc6i()) -
                    l.y * (1.0f / 6.0f) * (ri6 - g.rc6i());
        a.fe += in ? 0.5f * (uc + ulj) : 0.0f;
    }
}

/* Lane sums of two entries at a time (even and odd entries of a batch). */
template <bool PACKED>
struct pair_acc2 {
    v2<PACKED> fx, fy, fz, fw;
};

/* The minimum-image constants as register pairs (the same value in both
 * halves), so the shift of two entries is four packed instructions per axis:
 * d - L rint(d / L) with rint done by adding and subtracting 1.5 * 2^23.
 * The code generator may contract the packed multiply and the first add into
 * one FMA, rounding d / L + 1.5 * 2^23 once; that changes the shift only
 * where d / L lies within an ulp of a half-integer, i.e. |d| = L/2 to
 * 1e-5 A, and such a pair is beyond rc (< L/2) with either shift. */
template <bool PACKED>
struct wrap2 {
    v2<PACKED> li[3], nl[3], magic;
    template <class G>
    __device__ __forceinline__ static wrap2 make(const G &g)
    {
        wrap2 w;
        for (int d = 0; d < 3; d++) {
            w.li[d] = v2<PACKED>::make(g.Li(d), g.Li(d));
            w.nl[d] = v2<PACKED>::make(-g.L(d), -g.L(d));
        }
        w.magic = v2<PACKED>::make(12582912.0f, 12582912.0f);
        return w;
    }
    __device__ __forceinline__ v2<PACKED> shift(int d, v2<PACKED> x) const
    {
        const v2<PACKED> r = (x * li[d] + magic) - magic;
        return v2<PACKED>::fma(nl[d], r, x);
    }
};

/* Two pairs (i, j0) and (i, j1) at once: the operations whose operands all
 * vary per entry run on v2; those with a per-atom or per-system constant run
 * as scalar IEEE operations with the constant (no register pair to hold it).
 * The same formulas as pair_term, with every rounding step fixed. */
template <int KIND, bool WRAP, bool PACKED, class G>
__device__ __forceinline__ void pair_term2(const G &g, const wrap2<PACKED> &W, v2<PACKED> PX, v2<PACKED> PY,
                                           v2<PACKED> PZ, float qi, float4 p0, float4 p1, float2 l0,
                                           float2 l1, pair_acc2<PACKED> &a)
{
    typedef v2<PACKED> V;
    V dx = PX - V::make(p0.x, p1.x), dy = PY - V::make(p0.y, p1.y), dz = PZ - V::make(p0.z, p1.z);
    if (WRAP) {
        dx = W.shift(0, dx);
        dy = W.shift(1, dy);
        dz = W.shift(2, dz);
    }
    const V rsq = V::fma(dz, dz, V::fma(dy, dy, dx * dx));
    float s0, s1;
    rsq.get(s0, s1);
    const V ri = V::make(rsqrt_approx(s0), rsqrt_approx(s1));
    const V ri2 = ri * ri;
    const V qq = V::make(__fmul_rn(qi, p0.w), __fmul_rn(qi, p1.w));
    V ff;
    if (KIND == 1) {
        float r0, r1;
        (rsq * ri).get(r0, r1);
        const float t0 = rcp_approx(__fmaf_rn(g.palfa(), r0, 1.0f));
        const float t1 = rcp_approx(__fmaf_rn(g.palfa(), r1, 1.0f));
        const float e0 = ex2_approx(__fmul_rn(g.alfasq(), s0)), e1 = ex2_approx(__fmul_rn(g.alfasq(), s1));
        const float q0 = __fmul_rn(__fmaf_rn(__fmaf_rn(__fmaf_rn(__fmaf_rn(A5, t0, A4), t0, A3), t0, A2), t0, A1), t0);
        const float q1 = __fmul_rn(__fmaf_rn(__fmaf_rn(__fmaf_rn(__fmaf_rn(A5, t1, A4), t1, A3), t1, A2), t1, A1), t1);
        const V h = V::make(__fmaf_rn(g.spiialfa(), r0, q0), __fmaf_rn(g.spiialfa(), r1, q1));
        float h0, h1;
        (h * V::make(e0, e1) * ri).get(h0, h1);
        ff = V::make(__fsub_rn(h0, g.wolf()), __fsub_rn(h1, g.wolf())) * qq;
    } else {
        float a0, a1;
        ri.get(a0, a1);
        ff = qq * V::make(__fmaf_rn(-g.reacf(), s0, a0), __fmaf_rn(-g.reacf(), s1, a1));
    }
    const V ri6 = ri2 * ri2 * ri2;
    float m0, m1;
    ri6.get(m0, m1);
    const V lj = V::make(__fmaf_rn(l0.x, m0, -l0.y), __fmaf_rn(l1.x, m1, -l1.y)) * ri6 * ri2;
    ff = V::fma(ff, ri2, lj);
    /* list padding entries point at the atom itself: r = 0 is skipped */
    float f0, f1;
    ff.get(f0, f1);
    f0 = (s0 <= g.rcsq() && s0 > 0.0f) ? f0 : 0.0f;
    f1 = (s1 <= g.rcsq() && s1 > 0.0f) ? f1 : 0.0f;
    ff = V::make(f0, f1);
    a.fx = V::fma(ff, dx, a.fx);
    a.fy = V::fma(ff, dy, a.fy);
    a.fz = V::fma(ff, dz, a.fz);
    a.fw = V::fma(ff, rsq, a.fw);
}

struct pair_total {
    long long fx, fy, fz;   /* int64 fixed point, valid in lane 0 of the atom's group */
    float fw, fe;
};

/* Whether atom i sits at least rc (plus 0.1% of the box) from every face of
 * the box.  When every position lies in [-L/2, L/2] (G::centered()), for
 * such an atom every j within rc in the minimum image is within rc without
 * a shift: x_i - x_j needs no wrap, and equals the shifted difference bit
 * for bit (the shift there is L * 0).  A pair the unshifted difference puts
 * beyond L/2 on some axis is beyond rc (rc < L/2) and is dropped either way. */
template <class G>
__device__ __forceinline__ bool interior(const G &g, float4 pi)
{
    const float rc = sqrtf(g.rcsq());
    return fabsf(pi.x) + rc < 0.499f * g.L(0) && fabsf(pi.y) + rc < 0.499f * g.L(1) &&
           fabsf(pi.z) + rc < 0.499f * g.L(2);
}

/* The entries of one lane in batches of B, software pipelined: while batch
 * t is computed, the positions of batch t+1 and the list entries of batch
 * t+2 are in flight.  ljrow may point into shared memory (a batch's
 * per-replica table): plain loads there, not the read-only global path. */
template <int KIND, int TPA, int B, bool ENERGY, bool WRAP, bool PACK, int UNROLL, class G>
__device__ __forceinline__ void pair_loop(const G &g, float4 pi, float qi, int nb,
                                          const unsigned *__restrict__ lp,
                                          const float4 *__restrict__ pos4, const float2 *ljrow,
                                          pair_acc &acc)
{
    unsigned e0[B], e1[B];
    float4 p0[B];
    typedef v2<true> V;   /* used when PACK */
    const V PX = V::make(pi.x, pi.x), PY = V::make(pi.y, pi.y), PZ = V::make(pi.z, pi.z);
    const V zero = V::make(0.0f, 0.0f);
    pair_acc2<true> acc2 = {zero, zero, zero, zero};
    wrap2<true> W;
    if (PACK && WRAP) W = wrap2<true>::make(g);
    const V PXY = V::make(pi.x, pi.y);
    wrapxy WXY;
    if (!(PACK && !ENERGY && B % 2 == 0) && WRAP) WXY = wrapxy::make(g);
#pragma unroll
    for (int b = 0; b < B; b++) e0[b] = __ldg(lp + b * TPA);
#pragma unroll
    for (int b = 0; b < B; b++) p0[b] = __ldg(pos4 + (e0[b] & MD_INDEX_MASK));
    if (nb > 1) {
#pragma unroll
        for (int b = 0; b < B; b++) e1[b] = __ldg(lp + (B + b) * TPA);
    }
#pragma unroll UNROLL
    for (int t = 0; t < nb; t++) {
        float4 p1[B];
        unsigned e2[B];
        if (t + 1 < nb) {
#pragma unroll
            for (int b = 0; b < B; b++) p1[b] = __ldg(pos4 + (e1[b] & MD_INDEX_MASK));
        }
        if (t + 2 < nb) {
#pragma unroll
            for (int b = 0; b < B; b++) e2[b] = __ldg(lp + ((t + 2) * B + b) * TPA);
        }
        if (PACK && !ENERGY && B % 2 == 0) {
#pragma unroll
            for (int b = 0; b < B; b += 2)
                pair_term2<KIND, WRAP, true>(g, W, PX, PY, PZ, qi, p0[b], p0[b + 1], ljrow[e0[b] >> MD_TYPE_SHIFT],
                                             ljrow[e0[b + 1] >> MD_TYPE_SHIFT], acc2);
        } else {
#pragma unroll
            for (int b = 0; b < B; b++)
                pair_term<KIND, ENERGY, WRAP>(g, WXY, PXY, pi, qi, p0[b], ljrow[e0[b] >> MD_TYPE_SHIFT], true,
                                              acc);
        }
#pragma unroll
        for (int b = 0; b < B; b++) {
            e0[b] = e1[b];
            p0[b] = p1[b];
            e1[b] = e2[b];
        }
    }
    if (PACK && !ENERGY && B % 2 == 0) {
        float a0, a1;
        acc2.fx.get(a0, a1);
        acc.fx = __fadd_rn(a0, a1);
        acc2.fy.get(a0, a1);
        acc.fy = __fadd_rn(a0, a1);
        acc2.fz.get(a0, a1);
        acc.fz = __fadd_rn(a0, a1);
        acc2.fw.get(a0, a1);
        acc.fw = __fadd_rn(a0, a1);
    }
}

/* Pair forces of atom ii from its list: TPA lanes per atom, lane l takes the
 * entries l, l+TPA, ... in batches of B (TPA*B divides 32, the padding
 * quantum of the list rows, so no entry needs a bounds test).  A warp whose
 * atoms are all interior() skips the minimum-image shifts.  With PACK,
 * without energies and with even B, entries go two at a time through
 * pair_term2 as packed f32x2 instructions (each lane keeping even- and
 * odd-entry sums); otherwise one at a time through pair_term.  Each lane sums in
 * FP32 and converts its sum to int64 once; lane sums are combined with
 * integer shuffles (exact), so the result depends only on TPA.  Every lane of
 * the warp must call this (the shuffles use the full mask). */
template <int KIND, int TPA, int B, bool ENERGY, bool PACK = true, int UNROLL = 0, class G>
__device__ __forceinline__ pair_total pair_sum(const G &g, int cap, int ii, bool active, int lane,
                                               const float4 *__restrict__ pos4,
                                               const int *__restrict__ type,
                                               const unsigned *__restrict__ nl,
                                               const int *__restrict__ nl_n, const float2 *lj)
{
    static_assert(MD_LIST_QUANTUM % (TPA * B) == 0, "batch must divide the list padding");
    const float4 pi = pos4[ii];
    const int cnt = active ? nl_n[ii] : 0;
    /* unrolling of the batch loop (0: the packed loop rolled, which measured
     * fastest for a single system, 43 against 46 us per launch on 64000
     * ions; the scalar one twice) */
    constexpr int UNR = UNROLL ? UNROLL : ((PACK && !ENERGY && B % 2 == 0) ? 1 : 2);
    /* batches of TPA * B entries up to the first that holds the row's last
     * entry: the row is padded to a multiple of 32 (>= TPA * B) with entries
     * that add exactly zero, so the padding past that batch is skipped.  An
     * unrolled loop takes whole unrolled rounds where the padding holds
     * them (an odd count in some of a warp's rows made the unrolled loop's
     * remainder run as an extra pass: 1.58 against 1.46 ms per launch on the
     * 512-replica batch) */
    constexpr int QE = (MD_LIST_QUANTUM % (TPA * B * UNR) == 0) ? TPA * B * UNR : TPA * B;
    const int nb = (cnt + QE - 1) / QE * (QE / (TPA * B));
    const float2 *ljrow = lj + type[ii] * MD_MAXTYPE;
    const float qi = QFAC * pi.w;
    pair_acc acc = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
    const unsigned *lp = nl + (size_t)ii * cap + lane;
    const bool inner = g.centered() && __all_sync(0xffffffffu, !active || interior(g, pi));
    if (nb > 0) {
        if (inner)
            pair_loop<KIND, TPA, B, ENERGY, false, PACK, UNR>(g, pi, qi, nb, lp, pos4, ljrow, acc);
        else
            pair_loop<KIND, TPA, B, ENERGY, true, PACK, UNR>(g, pi, qi, nb, lp, pos4, ljrow, acc);
    }
    pair_total r;
    r.fx = __float2ll_rn(acc.fx * 4294967296.0f);
    r.fy = __float2ll_rn(acc.fy * 4294967296.0f);
    r.fz = __float2ll_rn(acc.fz * 4294967296.0f);
    r.fw = acc.fw;
    r.fe = acc.fe;
    if (TPA > 1) {
        const unsigned mask = 0xffffffffu;
#pragma unroll
        for (int off = TPA / 2; off > 0; off >>= 1) {
            r.fx += __shfl_down_sync(mask, r.fx, off, TPA);
            r.fy += __shfl_down_sync(mask, r.fy, off, TPA);
            r.fz += __shfl_down_sync(mask, r.fz, off, TPA);
            r.fw += __shfl_down_sync(mask, r.fw, off, TPA);
            if (ENERGY) r.fe += __shfl_down_sync(mask, r.fe, off, TPA);
        }
    }
    return r;
}

inline pair_consts make_pair_consts(const md_ctx *c)
{
    pair_consts pc;
    md_shift_consts(c->lkspace, c->rcutsq, c->alfa, c->reacf, &pc.ucc, &pc.rc6i, &pc.rcinv);
    return pc;
}

}  // namespace

#endif
