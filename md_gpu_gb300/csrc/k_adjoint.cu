/*
 * k_adjoint.cu -- gradients of trajectory-averaged observables of a batch
 * of replicas (velocity Verlet NVE) by the discrete adjoint, with
 * checkpoint-and-recompute.  No counterpart in the reference.
 *
 * Loss per replica (frames m = 0..K: the start and every step):
 *   L = w_pe <U>/N + w_rdf sum_b (gbar_b - t_b)^2,
 *   g_b(x) = V/(N_a N_b 4 pi r_b^2) sum_{i in a, j in b} K(r_b - r_ij),
 * K a normalised Gaussian of width sigma, r_b = (b + 1/2) dr, gbar the frame
 * average.  Gradients: every LJ table entry lj1[a][b], lj2[a][b] (as used by
 * the rows of atoms of type a) and the log of a common charge scale.
 *
 * Forward per step: v_h = v + c F(x); x' = x + dt v_h; v' = v_h + c F(x'),
 * c = dt/(2m).  Reverse mode with P = dL/dx and u_m = dL/dv_h(m):
 *   u_m = u_{m+1} + dt P_{m+1}                         (u_K = 0)
 *   P_m = P_{m+1} + dO_m/dx_m + f_m J(x_m) (c u_m)
 *   dL/dtheta += f_m (dF(x_m)/dtheta) . (c u_m) + dO_m/dtheta,
 * f_m = 2 for 0 < m < K (F(x_m) enters two half kicks with the same adjoint
 * vector), f_0 = 1; J = dF/dx is symmetric, for a pair potential
 *   (J w)_i = sum_j [ff (w_i - w_j) + g (d.(w_i - w_j)) d],  g = (dff/dr)/r.
 * The pair terms differentiate the force law the dynamics use (A&S 7.1.26
 * erfc included), in FP32, and so do the harmonic bonds and angles; the adjoint state P, u is FP64 in the original
 * atom order, and every sum is taken in a fixed order (block slots, then
 * replicas), so the gradient is deterministic.
 *
 * Checkpoints: (x, v) every C steps in the forward run.  The backward run
 * recomputes one segment of C steps at a time from its checkpoint, keeping
 * its positions, and sweeps the frames of the segment backwards.  Both runs
 * force a list build at every checkpoint frame, so the recomputed
 * trajectory is bit-identical to the forward one.
 */
#include <math.h>

#include <algorithm>
#include <vector>

#include "md_pair.cuh"
#include "md_thermo.cuh"

namespace {

constexpr int ADJ_TPA = 8;            /* lanes per atom in the adjoint pair kernels */
constexpr int ADJ_NA = MD_ADJ_ATOMS;  /* atoms per block (replica-aligned grid) */
constexpr int ADJ_THREADS = ADJ_NA * ADJ_TPA;
constexpr double ADJ_HFIX = 1048576.0; /* 2^20: fixed point of the RDF kernel values */

struct adj_par {
    int cap, pitch, nbins, rdf_a, rdf_b, with_w;
    float dr, sigma, inv_2s2, kn, rmaxsq, rdf_fac;
    float wpe_k;   /* w_pe / (K + 1): the PE weight of one frame, per atom over N */
    int tab_n;     /* points of the RDF-gradient table per replica */
    float tab_h, tab_hi;   /* its spacing (dr / 8) and inverse */
};

/* The RDF term of a pair's adjoint force at distance x:
 *   C(x) = sum_b s_b (x_b - x) exp(-(x_b - x)^2 / (2 sigma^2)),
 * over the bins whose centre x_b lies within 5 sigma of x (rdf_bins),
 * s_b = ebn[b].  It is fixed for the whole backward pass, so it is
 * tabulated once per replica, with its derivative
 *   C'(x) = sum_b s_b exp(-y^2 / (2 sigma^2)) (y^2 / sigma^2 - 1), y = x_b - x,
 * at spacing h = dr / 8, and read back by cubic Hermite interpolation
 * (error ~ (h / sigma)^4 / 384 of the term). */
__global__ void k_adj_rdf_table(adj_par ap, int nrep, const float *__restrict__ ebn, float2 *tab)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nrep * ap.tab_n) return;
    const int r = k / ap.tab_n, q = k - r * ap.tab_n;
    const double x = (double)q * ap.tab_h, dr = ap.dr, s = ap.sigma;
    const double reach = 5.0 * s, kk = 0.5 / (s * s);
    const int b0 = max((int)ceil((x - reach) / dr - 0.5), 0);
    const int b1 = min((int)floor((x + reach) / dr - 0.5), ap.nbins - 1);
    double c = 0.0, dc = 0.0;
    for (int b = b0; b <= b1; b++) {
        const double y = (b + 0.5) * dr - x, gq = exp(-y * y * kk), sb = ebn[(size_t)r * ap.nbins + b];
        c += sb * y * gq;
        dc += sb * gq * (2.0 * kk * y * y - 1.0);
    }
    tab[k] = make_float2((float)c, (float)dc);
}

/* C(r) from a replica's table (0 <= r < tab_h (tab_n - 1)). */
__device__ __forceinline__ float rdf_coef(const adj_par &ap, const float2 *__restrict__ tab, float r)
{
    const float u = r * ap.tab_hi;
    const int k = min((int)u, ap.tab_n - 2);
    const float t = u - (float)k, t2 = t * t, t3 = t2 * t;
    const float2 a = __ldg(tab + k), b = __ldg(tab + k + 1);
    const float h00 = 2.0f * t3 - 3.0f * t2 + 1.0f, h10 = t3 - 2.0f * t2 + t;
    const float h01 = 3.0f * t2 - 2.0f * t3, h11 = t3 - t2;
    return h00 * a.x + h01 * b.x + ap.tab_h * (h10 * a.y + h11 * b.y);
}

/* A row's per-neighbour-type parameter slots: lj1 terms, lj2 terms, then
 * the charge scale. */
template <int NT>
struct adj_slots {
    float p1[NT], p2[NT], ps;
};

/* exp(-y_b^2 / (2 sigma^2)) on the equally spaced bins y_b = y0 + (b - b0) dr by
 * the exact recurrence G(y + dr) = G(y) R(y), R(y + dr) = R(y) C with
 * R(y) = exp(-(2 y dr + dr^2) k), C = exp(-2 dr^2 k), k = 1/(2 sigma^2):
 * two exponentials per pair instead of one per bin. */
struct gauss_walk {
    float g, rr, c;
    __device__ __forceinline__ gauss_walk(float y0, float dr, float k, float cstep)
    {
        g = __expf(-y0 * y0 * k);
        rr = __expf(-(2.0f * y0 * dr + dr * dr) * k);
        c = cstep;
    }
    __device__ __forceinline__ void next()
    {
        g *= rr;
        rr *= c;
    }
};

/* Bins whose centre lies within 5 sigma of r. */
__device__ __forceinline__ void rdf_bins(const adj_par &ap, float r, int &b0, int &b1)
{
    const float reach = 5.0f * ap.sigma;
    b0 = max((int)ceilf((r - reach) / ap.dr - 0.5f), 0);
    b1 = min((int)floorf((r + reach) / ap.dr - 0.5f), ap.nbins - 1);
}

/* RDF histogram of one frame: every unordered (a, b) pair inside rmax is
 * counted once, by the row of its lower (sorted) index, so rows of both
 * types share the work (an (a, a) pair counts twice, as the ordered sum over
 * i in a, j in b does).  Kernel values in fixed point (2^-20) are summed with
 * integer atomics into per-warp histograms in shared memory, then added into
 * the replica's histogram.  The lanes of a warp first test their row
 * entries and queue the distances of the pairs that count (a quarter or
 * less of the entries) in shared memory; each full queue of 32 is deposited
 * with every lane busy. */
constexpr int ADJ_WARPS = ADJ_THREADS / 32;
constexpr int ADJ_RDF_BINS = 256;   /* per-warp histograms hold up to 256 bins */

__device__ __forceinline__ void rdf_deposit(const adj_par &ap, float r, float wt, float cstep,
                                            unsigned *h)
{
    int b0, b1;
    rdf_bins(ap, r, b0, b1);
    gauss_walk gw(((float)b0 + 0.5f) * ap.dr - r, ap.dr, ap.inv_2s2, cstep);
    for (int b = b0; b <= b1; b++) {
        /* <= 1.7e7 per pair and bin; a warp's bin stays far below 2^32 per frame */
        atomicAdd(&h[b], __float2uint_rn(wt * gw.g));
        gw.next();
    }
}

__global__ void __launch_bounds__(ADJ_THREADS) k_adj_rdf(adj_par ap, const int2 *__restrict__ tab,
                                                       const md_rep *__restrict__ reps,
                                                       const float4 *__restrict__ pos4,
                                                       const int *__restrict__ type,
                                                       const unsigned *__restrict__ nl,
                                                       const int *__restrict__ nl_n,
                                                       unsigned long long *hist)
{
    __shared__ unsigned s_h[ADJ_WARPS][ADJ_RDF_BINS];
    __shared__ float s_q[ADJ_WARPS][64];
    for (int k = threadIdx.x; k < ADJ_WARPS * ADJ_RDF_BINS; k += blockDim.x) (&s_h[0][0])[k] = 0u;
    __syncthreads();
    const int2 bt = tab[blockIdx.x];
    const md_rep &R = reps[bt.x];
    const geom_reg g = rep_geom(R);
    const int a = threadIdx.x / ADJ_TPA, lane = threadIdx.x % ADJ_TPA, w = threadIdx.x >> 5;
    const int wl = threadIdx.x & 31;
    const unsigned lt = (1u << wl) - 1u;
    const int i = bt.y + a;
    const float cstep = __expf(-2.0f * ap.dr * ap.dr * ap.inv_2s2);
    const int ti = i < R.atom0 + R.natom ? type[i] : -1;
    const int want = ti == ap.rdf_a ? ap.rdf_b : (ti == ap.rdf_b ? ap.rdf_a : -1);
    const float wt = ap.rdf_fac * ap.kn * (float)ADJ_HFIX;
    const float4 pi = want >= 0 ? pos4[i] : make_float4(0.f, 0.f, 0.f, 0.f);
    const int cnt = want >= 0 ? nl_n[i] : 0;
    int cmax = cnt;   /* the warp's longest row */
    for (int o = 16; o > 0; o >>= 1) cmax = max(cmax, __shfl_xor_sync(0xffffffffu, cmax, o));
    int fill = 0;
    for (int k0 = 0; k0 < cmax; k0 += ADJ_TPA) {
        const int k = k0 + lane;
        bool ok = false;
        float r = 0.0f;
        if (k < cnt) {
            const unsigned e = nl[(size_t)i * ap.cap + k];
            const int j = (int)(e & MD_INDEX_MASK);
            if ((int)(e >> MD_TYPE_SHIFT) == want && j > i) {
                const float4 pj = pos4[j];
                float dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
                dx -= g.L(0) * rint_small(dx * g.Li(0));
                dy -= g.L(1) * rint_small(dy * g.Li(1));
                dz -= g.L(2) * rint_small(dz * g.Li(2));
                const float rsq = dx * dx + dy * dy + dz * dz;
                if (rsq < ap.rmaxsq) {
                    ok = true;
                    r = rsq * rsqrt_approx(rsq);
                }
            }
        }
        const unsigned bal = __ballot_sync(0xffffffffu, ok);
        if (ok) s_q[w][fill + __popc(bal & lt)] = r;
        fill += __popc(bal);
        __syncwarp();
        if (fill >= 32) {
            rdf_deposit(ap, s_q[w][wl], wt, cstep, s_h[w]);
            __syncwarp();
            const bool mv = wl < fill - 32;
            const float t = mv ? s_q[w][32 + wl] : 0.0f;
            __syncwarp();
            if (mv) s_q[w][wl] = t;
            fill -= 32;
            __syncwarp();
        }
    }
    if (wl < fill) rdf_deposit(ap, s_q[w][wl], wt, cstep, s_h[w]);
    __syncthreads();
    for (int k = threadIdx.x; k < ap.nbins; k += blockDim.x) {
        unsigned long long t = 0ull;
        for (int q = 0; q < ADJ_WARPS; q++) t += s_h[q][k];
        if (t) atomicAdd(&hist[(size_t)bt.x * ap.nbins + k], t);
    }
}

/* Per-replica sum of the frame's potential energies (from the last
 * velocity-Verlet reduction), one thread per replica. */
__global__ void k_adj_pe(int nrep, const md_repstate *__restrict__ repst, double *pe_sum)
{
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r < nrep) pe_sum[r] += repst[r].pe;
}

/* u += dt P (not at the last frame), w = f_m c u with c = dt/(2m) =
 * kick/2 * 2^32; sorted-order w4, original-order P and u (3 per atom). */
__global__ void k_adj_w(int n, double dt, int update, double fac, const int *__restrict__ perm,
                        const double *__restrict__ kick, double *U, const double *__restrict__ Pv,
                        float4 *w4)
{
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    const size_t o = 3 * (size_t)perm[s];
    const double c = fac * 0.5 * kick[s] * FX_SCALE;
    double u[3];
    for (int d = 0; d < 3; d++) {
        u[d] = U[o + d];
        if (update) {
            u[d] += dt * Pv[o + d];
            U[o + d] = u[d];
        }
    }
    w4[s] = make_float4((float)(c * u[0]), (float)(c * u[1]), (float)(c * u[2]), 0.0f);
}

/* P += G (sorted-order G, original-order P). */
__global__ void k_adj_acc(int n, int pitch, const int *__restrict__ perm, const double *__restrict__ G,
                          double *Pv)
{
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    const size_t o = 3 * (size_t)perm[s];
    for (int d = 0; d < 3; d++) Pv[o + d] += G[(size_t)d * pitch + s];
}

/* The bonded part of one frame's adjoint force, added to G after the pair
 * kernel: per sorted atom s, G_s += (J_b w)_s - wpe F_b,s for the harmonic
 * bonds and angles of k_bonded (bonded_forces.cu:34-193 as the dynamics
 * evaluate them, rsqrtf and acosf included).  (J_b w)_s is the derivative of
 * F_b,s along w: the same expressions carried with their first-order
 * variations (the minimum-image shift is constant; the clamp of cos(theta)
 * has zero variation where it clamps).  One thread per atom. */
__device__ __forceinline__ void adj_min_image(float &x, float &y, float &z, const float *L, const float *Li)
{
    x -= L[0] * rintf(x * Li[0]);
    y -= L[1] * rintf(y * Li[1]);
    z -= L[2] * rintf(z * Li[2]);
}

__global__ void k_adj_bonded(int n, int pitch, adj_par ap, const md_rep *__restrict__ reps,
                             const int *__restrict__ arep, const float4 *__restrict__ pos4,
                             const float4 *__restrict__ w4, const int2 *__restrict__ bl_s,
                             const int *__restrict__ bl_sn, const int4 *__restrict__ al_s,
                             const int *__restrict__ al_sn, const float *__restrict__ par, int has_bonds,
                             int has_angles, double *G)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    const int nb = has_bonds ? bl_sn[s] : 0, na = has_angles ? al_sn[s] : 0;
    if (nb == 0 && na == 0) return;
    const md_rep &R = reps[arep[s]];
    const float wpe = ap.wpe_k / (float)R.natom;
    const float *bnd1 = par, *bnd2 = par + MD_MAXTYPE, *ang1 = par + 2 * MD_MAXTYPE,
                *ang2 = par + 3 * MD_MAXTYPE;
    const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
    auto wof = [&](int k) { return ap.with_w ? w4[k] : zero; };
    const float4 p = pos4[s], ws = wof(s);
    float fx = 0.f, fy = 0.f, fz = 0.f, tx = 0.f, ty = 0.f, tz = 0.f;
    for (int k = 0; k < nb; k++) {
        const int2 b = bl_s[(size_t)k * pitch + s];
        const float4 q = pos4[b.x], wq = wof(b.x);
        float dx = p.x - q.x, dy = p.y - q.y, dz = p.z - q.z;
        adj_min_image(dx, dy, dz, R.box, R.boxi);
        const float ux = ws.x - wq.x, uy = ws.y - wq.y, uz = ws.z - wq.z;
        const float rsq = dx * dx + dy * dy + dz * dz;
        const float ri = rsqrtf(rsq);
        const float kk = bnd1[b.y], r0 = bnd2[b.y];
        const float fa = kk * (r0 * ri - 1.0f);
        const float ri_t = -ri * ri * ri * (dx * ux + dy * uy + dz * uz);
        const float fa_t = kk * r0 * ri_t;
        fx += fa * dx; fy += fa * dy; fz += fa * dz;
        tx += fa_t * dx + fa * ux; ty += fa_t * dy + fa * uy; tz += fa_t * dz + fa * uz;
    }
    for (int k = 0; k < na; k++) {
        const int4 a = al_s[(size_t)k * pitch + s];
        const float4 qb = pos4[a.z], wb = wof(a.z);
        float4 qa, cen, wa, wc;
        if (a.x == 1) { qa = pos4[a.y]; wa = wof(a.y); cen = p; wc = ws; }   /* this atom is the centre */
        else { qa = p; wa = ws; cen = pos4[a.y]; wc = wof(a.y); }           /* this atom is an end */
        float ax = qa.x - cen.x, ay = qa.y - cen.y, az = qa.z - cen.z;
        adj_min_image(ax, ay, az, R.box, R.boxi);
        float bx = qb.x - cen.x, by = qb.y - cen.y, bz = qb.z - cen.z;
        adj_min_image(bx, by, bz, R.box, R.boxi);
        const float tax = wa.x - wc.x, tay = wa.y - wc.y, taz = wa.z - wc.z;
        const float tbx = wb.x - wc.x, tby = wb.y - wc.y, tbz = wb.z - wc.z;
        const float ai = rsqrtf(ax * ax + ay * ay + az * az);
        const float bi = rsqrtf(bx * bx + by * by + bz * bz);
        const float ai_t = -ai * ai * ai * (ax * tax + ay * tay + az * taz);
        const float bi_t = -bi * bi * bi * (bx * tbx + by * tby + bz * tbz);
        const float ab = ax * bx + ay * by + az * bz;
        const float ab_t = tax * bx + tay * by + taz * bz + ax * tbx + ay * tby + az * tbz;
        const float c0 = ab * ai * bi;
        const float cang = fminf(fmaxf(c0, -0.9999999f), 0.9999999f);
        const float c_t = cang == c0 ? ab_t * ai * bi + ab * ai_t * bi + ab * ai * bi_t : 0.0f;
        const float th = acosf(cang);
        const float s1 = rsqrtf(1.0f - cang * cang);
        const float th_t = -c_t * s1;
        const float s1_t = s1 * s1 * s1 * cang * c_t;
        const float k1 = ang1[a.w], th0 = ang2[a.w];
        const float ff = k1 * (th - th0) * s1 * ai * bi;
        const float ff_t =
            k1 * (th_t * s1 * ai * bi + (th - th0) * (s1_t * ai * bi + s1 * ai_t * bi + s1 * ai * bi_t));
        const float aa = ab * ai * ai, aa_t = ab_t * ai * ai + 2.0f * ab * ai * ai_t;
        float gx = bx - aa * ax, gy = by - aa * ay, gz = bz - aa * az;
        float gx_t = tbx - aa_t * ax - aa * tax, gy_t = tby - aa_t * ay - aa * tay,
              gz_t = tbz - aa_t * az - aa * taz;
        if (a.x == 1) {
            const float bb = ab * bi * bi, bb_t = ab_t * bi * bi + 2.0f * ab * bi * bi_t;
            gx = bb * bx - ax - gx;
            gy = bb * by - ay - gy;
            gz = bb * bz - az - gz;
            gx_t = bb_t * bx + bb * tbx - tax - gx_t;
            gy_t = bb_t * by + bb * tby - tay - gy_t;
            gz_t = bb_t * bz + bb * tbz - taz - gz_t;
        }
        fx += ff * gx; fy += ff * gy; fz += ff * gz;
        tx += ff_t * gx + ff * gx_t; ty += ff_t * gy + ff * gy_t; tz += ff_t * gz + ff * gz_t;
    }
    G[s] += (double)tx - (double)(wpe * fx);
    G[(size_t)pitch + s] += (double)ty - (double)(wpe * fy);
    G[2 * (size_t)pitch + s] += (double)tz - (double)(wpe * fz);
}

/* The adjoint pair kernel of one frame: per atom i (ADJ_TPA lanes over its
 * list row) G_i = J(x) w |_i - wpe F_i + d(sum_b e_b g_b)/dx_i, and the
 * row's parameter slots; the block reduces its rows into (type, slot) sums
 * in a fixed order.  ebn[b] = e_b norm_b kn / sigma^2 of the replica. */
template <int KIND, int NT>
__global__ void __launch_bounds__(ADJ_THREADS) k_adj_back(
    adj_par ap, const int2 *__restrict__ tab, const md_rep *__restrict__ reps,
    const float2 *__restrict__ ljr, const float2 *__restrict__ rtab, const float4 *__restrict__ pos4,
    const int *__restrict__ type, const unsigned *__restrict__ nl, const int *__restrict__ nl_n,
    const float4 *__restrict__ w4, double *G, double *part)
{
    constexpr int NS = 2 * NT + 1;           /* slots of a row */
    constexpr int NB = 2 * NT * NT + 1;      /* slots of a block: (type, slot) */
    __shared__ float2 lj[MD_MAXTYPE * MD_MAXTYPE];
    __shared__ float s_val[ADJ_NA][NS];
    __shared__ int s_type[ADJ_NA];
    const int2 bt = tab[blockIdx.x];
    const md_rep &R = reps[bt.x];
    if (threadIdx.x < MD_MAXTYPE * MD_MAXTYPE)
        lj[threadIdx.x] = ljr[bt.x * MD_MAXTYPE * MD_MAXTYPE + threadIdx.x];
    const geom_reg g = rep_geom(R);
    const float wpe = ap.wpe_k / (float)R.natom;
    const float W = R.wolf, A = R.palfa;
    const float spi = R.spiialfa;
    const float alsq = -R.alfasq * 0.69314718f;   /* alpha^2 (alfasq = -alpha^2 / ln 2) */
    __syncthreads();
    const int a = threadIdx.x / ADJ_TPA, lane = threadIdx.x % ADJ_TPA;
    const int i = bt.y + a;
    const bool active = i < R.atom0 + R.natom;
    const int ii = active ? i : bt.y;
    const float4 pi = pos4[ii];
    const int ti = type[ii];
    const float qi = QFAC * pi.w;
    const float4 wi = ap.with_w ? w4[ii] : make_float4(0.f, 0.f, 0.f, 0.f);
    const bool ra = ti == ap.rdf_a, rb = ti == ap.rdf_b;
    const float2 *rt = rtab + (size_t)bt.x * ap.tab_n;
    float gx = 0.f, gy = 0.f, gz = 0.f;
    adj_slots<NT> sl;
#pragma unroll
    for (int k = 0; k < NT; k++) { sl.p1[k] = 0.f; sl.p2[k] = 0.f; }
    sl.ps = 0.f;
    const int cnt = active ? nl_n[ii] : 0;
    const unsigned *row = nl + (size_t)ii * ap.cap;
    /* the next entry's position and w are loaded while this one is computed */
    unsigned en = lane < cnt ? row[lane] : 0u;
    float4 pn = pos4[lane < cnt ? (int)(en & MD_INDEX_MASK) : ii];
    float4 wn = ap.with_w && lane < cnt ? w4[en & MD_INDEX_MASK] : make_float4(0.f, 0.f, 0.f, 0.f);
    for (int k = lane; k < cnt; k += ADJ_TPA) {
        const unsigned e = en;
        const float4 pj = pn;
        const float4 wj = wn;
        if (k + ADJ_TPA < cnt) {
            en = row[k + ADJ_TPA];
            pn = pos4[en & MD_INDEX_MASK];
            if (ap.with_w) wn = w4[en & MD_INDEX_MASK];
        }
        const int tj = (int)(e >> MD_TYPE_SHIFT);
        float dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
        dx -= g.L(0) * rint_small(dx * g.Li(0));
        dy -= g.L(1) * rint_small(dy * g.Li(1));
        dz -= g.L(2) * rint_small(dz * g.Li(2));
        const float rsq = dx * dx + dy * dy + dz * dz;
        if (rsq > g.rcsq() || rsq == 0.0f) continue;
        /* the approximations the dynamics use (PTX rsqrt/rcp/ex2.approx) */
        const float ri = rsqrt_approx(rsq), r = rsq * ri, ri2 = ri * ri;
        const float qq = qi * pj.w;
        float fc, dfc, uc;
        if (KIND == 1) {
            const float t = rcp_approx(1.0f + A * r);
            const float P = (((A5 * t + A4) * t + A3) * t + A2) * t + A1;
            const float dPt = (((5.0f * A5 * t + 4.0f * A4) * t + 3.0f * A3) * t + 2.0f * A2) * t + A1;
            const float ex = ex2_approx(R.alfasq * rsq);
            const float E = P * t * ex;
            const float dE = -dPt * A * t * t * ex - 2.0f * alsq * r * E;
            const float h = spi * ex + E * ri;
            const float dh = -2.0f * alsq * r * spi * ex + dE * ri - E * ri2;
            fc = qq * (h - W) * ri2;
            dfc = qq * (dh * ri2 - 2.0f * (h - W) * ri2 * ri);
            uc = qq * (E * ri - g.ucc() + W * __logf(r * g.rcinv()));
        } else {
            fc = qq * (ri * ri2 - g.reacf());
            dfc = -3.0f * qq * ri2 * ri2;
            uc = qq * (ri + 0.5f * g.reacf() * rsq - g.ucc());
        }
        const float2 l = lj[ti * MD_MAXTYPE + tj];
        const float ri6 = ri2 * ri2 * ri2, ri8 = ri6 * ri2, ri14 = ri6 * ri8;
        const float ff = fc + l.x * ri14 - l.y * ri8;
        const float gg = (dfc - 14.0f * l.x * ri14 * ri + 8.0f * l.y * ri8 * ri) * ri;
        /* observable: - wpe F_i */
        gx -= wpe * ff * dx;
        gy -= wpe * ff * dy;
        gz -= wpe * ff * dz;
        float dwi = 0.0f;
        if (ap.with_w) {
            const float ux = wi.x - wj.x, uy = wi.y - wj.y, uz = wi.z - wj.z;
            const float dd = dx * ux + dy * uy + dz * uz;
            gx += ff * ux + gg * dd * dx;
            gy += ff * uy + gg * dd * dy;
            gz += ff * uz + gg * dd * dz;
            dwi = dx * wi.x + dy * wi.y + dz * wi.z;
        }
        /* RDF pairs (a, b) in either orientation */
        if (((ra && tj == ap.rdf_b) || (rb && tj == ap.rdf_a)) && rsq < ap.rmaxsq) {
            const float coef = rdf_coef(ap, rt, r) * ap.rdf_fac * ri;
            gx += coef * dx;
            gy += coef * dy;
            gz += coef * dz;
        }
        /* parameter slots: dynamics (d.w_i) and the explicit PE derivative
         * (half of the pair's energy belongs to this row) */
        const float rc6i = g.rc6i();
        const float v1 = ri14 * dwi + 0.5f * wpe * (ri6 * ri6 - rc6i * rc6i) * (1.0f / 12.0f);
        const float v2 = -ri8 * dwi - 0.5f * wpe * (ri6 - rc6i) * (1.0f / 6.0f);
#pragma unroll
        for (int q = 0; q < NT; q++) {
            sl.p1[q] += q == tj ? v1 : 0.0f;
            sl.p2[q] += q == tj ? v2 : 0.0f;
        }
        sl.ps += 2.0f * fc * dwi + wpe * uc;
    }
    /* combine the lanes of the row (fixed order) */
#pragma unroll
    for (int off = ADJ_TPA / 2; off > 0; off >>= 1) {
        gx += __shfl_down_sync(0xffffffffu, gx, off, ADJ_TPA);
        gy += __shfl_down_sync(0xffffffffu, gy, off, ADJ_TPA);
        gz += __shfl_down_sync(0xffffffffu, gz, off, ADJ_TPA);
#pragma unroll
        for (int q = 0; q < NT; q++) {
            sl.p1[q] += __shfl_down_sync(0xffffffffu, sl.p1[q], off, ADJ_TPA);
            sl.p2[q] += __shfl_down_sync(0xffffffffu, sl.p2[q], off, ADJ_TPA);
        }
        sl.ps += __shfl_down_sync(0xffffffffu, sl.ps, off, ADJ_TPA);
    }
    if (lane == 0) {
        if (active) {
            const size_t P = (size_t)ap.pitch;
            G[i] = gx;
            G[P + i] = gy;
            G[2 * P + i] = gz;
        }
#pragma unroll
        for (int q = 0; q < NT; q++) {
            s_val[a][q] = active ? sl.p1[q] : 0.0f;
            s_val[a][NT + q] = active ? sl.p2[q] : 0.0f;
        }
        s_val[a][2 * NT] = active ? sl.ps : 0.0f;
        s_type[a] = active ? ti : -1;
    }
    __syncthreads();
    /* block slots: (row type, neighbour type, lj1 | lj2) and the charge
     * scale, each summed over the block's rows in order */
    if (threadIdx.x < NB) {
        const int k = threadIdx.x;
        double acc = 0.0;
        if (k == NB - 1) {
            for (int r2 = 0; r2 < ADJ_NA; r2++) acc += (double)s_val[r2][2 * NT];
        } else {
            const int tt = k / (2 * NT), rem = k % (2 * NT);   /* row type, slot */
            for (int r2 = 0; r2 < ADJ_NA; r2++)
                if (s_type[r2] == tt) acc += (double)s_val[r2][rem];
        }
        part[(size_t)blockIdx.x * NB + k] = acc;
    }
}

/* Per replica and block slot (one warp each): the replica's blocks summed
 * lane-strided, then by a fixed shuffle tree, added to its gradient
 * accumulators. */
__global__ void k_adj_param(int nrep, int nb_slots, const md_rep *__restrict__ reps,
                            const double *__restrict__ part, double *acc)
{
    const int t = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (t >= nrep * nb_slots) return;
    const int r = t / nb_slots, k = t % nb_slots;
    const md_rep &R = reps[r];
    double s = 0.0;
    for (int b = lane; b < R.anblk; b += 32) s += part[(size_t)(R.ablk0 + b) * nb_slots + k];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if (lane == 0) acc[t] += s;
}

template <int KIND, int NT>
void launch_back_nt(md_ctx *c, const adj_par &ap, const float2 *rtab, const float4 *w4, double *G,
                    double *part)
{
    const int k = md_grid_index(ADJ_NA);
    k_adj_back<KIND, NT><<<c->grid_cnt[k], ADJ_THREADS, 0, c->stream>>>(
        ap, c->grid_tab + c->grid_off[k], c->reps_dev, c->ljr_dev, rtab, c->pos4, c->type, c->nl,
        c->nl_n, w4, G, part);
}

int adj_nt(int ntype) { return ntype <= 1 ? 1 : (ntype <= 2 ? 2 : (ntype <= 4 ? 4 : 8)); }

void launch_back(md_ctx *c, const adj_par &ap, const float2 *rtab, const float4 *w4, double *G,
                 double *part)
{
    const int nt = adj_nt(c->ntype);
#define MD_ADJ_NT(K, N) \
    if (c->lkspace == K && nt == N) { launch_back_nt<K == 0 ? 0 : 1, N>(c, ap, rtab, w4, G, part); return; }
    MD_ADJ_NT(0, 1) MD_ADJ_NT(0, 2) MD_ADJ_NT(0, 4) MD_ADJ_NT(0, 8)
    MD_ADJ_NT(1, 1) MD_ADJ_NT(1, 2) MD_ADJ_NT(1, 4) MD_ADJ_NT(1, 8)
    MD_ADJ_NT(2, 1) MD_ADJ_NT(2, 2) MD_ADJ_NT(2, 4) MD_ADJ_NT(2, 8)
#undef MD_ADJ_NT
}

/* Device buffers of one adjoint run. */
struct adj_buffers {
    double *ck_x = nullptr, *ck_v = nullptr;   /* checkpoints, original order (3n each) */
    double *seg = nullptr;                     /* positions of one segment's frames */
    double *xK = nullptr, *vK = nullptr;       /* the final state */
    double *P = nullptr, *U = nullptr, *G = nullptr, *pe_sum = nullptr, *part = nullptr,
           *acc = nullptr;
    float4 *w4 = nullptr;
    float *ebn = nullptr;
    float2 *rtab = nullptr;
    unsigned long long *hist = nullptr;
    ~adj_buffers()
    {
        void *p[] = {ck_x, ck_v, seg, xK, vK, P, U, G, pe_sum, part, acc, w4, ebn, rtab, hist};
        for (void *q : p)
            if (q) cudaFree(q);
    }
};

template <class T>
cudaError_t adj_alloc(T **p, size_t count)
{
    return cudaMalloc((void **)p, sizeof(T) * std::max<size_t>(count, 1));
}

}  // namespace

extern "C" md_status md_adjoint_run(md_ctx *c, const md_adjoint_cfg *cfg, const double *target,
                                    double *loss, double *gbar, double *dlj1, double *dlj2,
                                    double *dlns)
{
    if (!c || !cfg || !loss) return MD_ERR_ARG;
    if (!c->batch || c->integrator != MD_VV || c->enstype != 0 || c->fp64) {
        c->last_error = "md_adjoint_run: needs a batch context with velocity Verlet NVE in FP32 mode";
        return MD_ERR_UNSUPPORTED;
    }
    const int K = cfg->nsteps, C = cfg->checkpoint > 0 ? cfg->checkpoint : 50;
    const int nb = cfg->nbins, nrep = c->nrep, n = c->n;
    if (K < 1 || nb < 1 || nb > ADJ_RDF_BINS || cfg->rdf_dr <= 0 || cfg->rdf_sigma <= 0 ||
        cfg->rdf_a < 0 || cfg->rdf_b < 0 || cfg->rdf_a >= c->ntype || cfg->rdf_b >= c->ntype ||
        (cfg->gradient && (!dlj1 || !dlj2 || !dlns))) {
        c->last_error = "md_adjoint_run: invalid configuration";
        return MD_ERR_ARG;
    }
    const double rmax = nb * cfg->rdf_dr + 5.0 * cfg->rdf_sigma;
    for (const md_rep &R : c->reps)
        if (rmax * rmax > (double)R.rcutsq) {
            c->last_error = "md_adjoint_run: RDF range beyond a replica's cutoff";
            return MD_ERR_ARG;
        }
    const int nseg = (K + C - 1) / C;
    const int nt = adj_nt(c->ntype), NB = 2 * nt * nt + 1;
    const int kla = md_grid_index(ADJ_NA), nblk = c->grid_cnt[kla];
    adj_buffers B;
    MD_CUDA_TRY(c, adj_alloc(&B.ck_x, 3 * (size_t)n * (nseg + 1)));
    MD_CUDA_TRY(c, adj_alloc(&B.ck_v, 3 * (size_t)n * (nseg + 1)));
    MD_CUDA_TRY(c, adj_alloc(&B.seg, 3 * (size_t)n * (C + 1)));
    MD_CUDA_TRY(c, adj_alloc(&B.xK, 3 * (size_t)n));
    MD_CUDA_TRY(c, adj_alloc(&B.vK, 3 * (size_t)n));
    MD_CUDA_TRY(c, adj_alloc(&B.P, 3 * (size_t)n));
    MD_CUDA_TRY(c, adj_alloc(&B.U, 3 * (size_t)n));
    MD_CUDA_TRY(c, adj_alloc(&B.G, 3 * (size_t)c->pitch));
    MD_CUDA_TRY(c, adj_alloc(&B.pe_sum, nrep));
    MD_CUDA_TRY(c, adj_alloc(&B.part, (size_t)nblk * NB));
    MD_CUDA_TRY(c, adj_alloc(&B.acc, (size_t)nrep * NB));
    MD_CUDA_TRY(c, adj_alloc(&B.w4, c->pitch));
    MD_CUDA_TRY(c, adj_alloc(&B.ebn, (size_t)nrep * nb));
    const float tab_h = (float)(cfg->rdf_dr / 8.0);
    const int tab_n = (int)(rmax / (double)tab_h) + 3;   /* covers [0, rmax + h] */
    MD_CUDA_TRY(c, adj_alloc(&B.rtab, (size_t)nrep * tab_n));
    MD_CUDA_TRY(c, adj_alloc(&B.hist, (size_t)nrep * nb));
    cudaStream_t s = c->stream;
    MD_CUDA_TRY(c, cudaMemsetAsync(B.hist, 0, sizeof(unsigned long long) * nrep * nb, s));
    MD_CUDA_TRY(c, cudaMemsetAsync(B.pe_sum, 0, sizeof(double) * nrep, s));

    adj_par ap;
    ap.cap = c->cap;
    ap.pitch = c->pitch;
    ap.nbins = nb;
    ap.rdf_a = cfg->rdf_a;
    ap.rdf_b = cfg->rdf_b;
    ap.with_w = 0;
    ap.dr = (float)cfg->rdf_dr;
    ap.sigma = (float)cfg->rdf_sigma;
    ap.inv_2s2 = (float)(0.5 / (cfg->rdf_sigma * cfg->rdf_sigma));
    ap.kn = (float)(1.0 / (sqrt(2.0 * M_PI) * cfg->rdf_sigma));
    ap.rmaxsq = (float)(rmax * rmax);
    ap.rdf_fac = cfg->rdf_a == cfg->rdf_b ? 2.0f : 1.0f;
    ap.wpe_k = (float)(cfg->w_pe / (K + 1));
    ap.tab_h = tab_h;
    ap.tab_hi = 1.0f / tab_h;
    ap.tab_n = tab_n;
    const int rgrid = (nrep + 255) / 256;
    const int agrid = (n + 255) / 256;

    md_kparams kp = md_make_kparams(c);
    auto obs = [&]() {
        k_adj_rdf<<<nblk, ADJ_THREADS, 0, s>>>(ap, c->grid_tab + c->grid_off[kla], c->reps_dev,
                                                  c->pos4, c->type, c->nl, c->nl_n, B.hist);
        k_adj_pe<<<rgrid, 256, 0, s>>>(nrep, c->repst, B.pe_sum);
    };
    auto save = [&](double *x, double *v) {
        launch_gather_out(c, kp, 0, c->io_dev);
        cudaMemcpyAsync(x, c->io_dev, sizeof(double) * 3 * n, cudaMemcpyDeviceToDevice, s);
        if (v) {
            launch_gather_out(c, kp, 1, c->io_dev);
            cudaMemcpyAsync(v, c->io_dev, sizeof(double) * 3 * n, cudaMemcpyDeviceToDevice, s);
        }
    };
    /* one VV step, the list forced at checkpoint frames */
    auto step = [&](int s_idx) {
        launch_vv_first(c, kp, 0, 0);
        launch_rebuild(c, kp, (s_idx + 1) % C == 0, (s_idx + 1) % C == 0);
        launch_forces(c, kp, true, MD_TERM_ALL);
        launch_vv_second(c, kp, 1);
    };

    /* ---- forward ---- */
    launch_rebuild(c, kp, true, true);
    launch_forces(c, kp, true, MD_TERM_ALL);
    launch_thermo_from_state(c, kp, 1);
    obs();
    save(B.ck_x, B.ck_v);
    for (int st = 0; st < K; st++) {
        step(st);
        obs();
        if ((st + 1) % C == 0) save(B.ck_x + 3 * (size_t)n * ((st + 1) / C), B.ck_v + 3 * (size_t)n * ((st + 1) / C));
    }
    save(B.xK, B.vK);
    std::vector<unsigned long long> hh((size_t)nrep * nb);
    std::vector<double> pes(nrep);
    MD_CUDA_TRY(c, cudaMemcpyAsync(hh.data(), B.hist, sizeof(unsigned long long) * hh.size(),
                                   cudaMemcpyDeviceToHost, s));
    MD_CUDA_TRY(c, cudaMemcpyAsync(pes.data(), B.pe_sum, sizeof(double) * nrep, cudaMemcpyDeviceToHost, s));
    MD_CUDA_TRY(c, cudaStreamSynchronize(s));
    MD_CUDA_TRY(c, cudaGetLastError());
    std::vector<float> ebn((size_t)nrep * nb);
    for (int r = 0; r < nrep; r++) {
        const md_rep &R = c->reps[r];
        int na = 0, nbt = 0;
        for (int i = 0; i < R.natom; i++) {
            na += c->itype[R.atom0 + i] == cfg->rdf_a;
            nbt += c->itype[R.atom0 + i] == cfg->rdf_b;
        }
        const double V = (double)R.box[0] * R.box[1] * R.box[2];
        double L = cfg->w_pe * pes[r] / (K + 1) / R.natom;
        for (int b = 0; b < nb; b++) {
            const double rb = (b + 0.5) * cfg->rdf_dr;
            const double norm = (na > 0 && nbt > 0) ? V / ((double)na * nbt * 4.0 * M_PI * rb * rb) : 0.0;
            const double g = norm * (double)hh[(size_t)r * nb + b] / ADJ_HFIX / (K + 1);
            const double t = target ? target[(size_t)r * nb + b] : 0.0;
            L += cfg->w_rdf * (g - t) * (g - t);
            if (gbar) gbar[(size_t)r * nb + b] = g;
            const double e = cfg->w_rdf * 2.0 * (g - t) / (K + 1);
            ebn[(size_t)r * nb + b] = (float)(e * norm / (sqrt(2.0 * M_PI) * cfg->rdf_sigma) /
                                              (cfg->rdf_sigma * cfg->rdf_sigma));
        }
        loss[r] = L;
    }
    if (!cfg->gradient) return MD_OK;

    /* ---- backward ---- */
    MD_CUDA_TRY(c, cudaMemcpyAsync(B.ebn, ebn.data(), sizeof(float) * ebn.size(), cudaMemcpyHostToDevice, s));
    k_adj_rdf_table<<<(nrep * ap.tab_n + 255) / 256, 256, 0, s>>>(ap, nrep, B.ebn, B.rtab);
    MD_CUDA_TRY(c, cudaMemsetAsync(B.P, 0, sizeof(double) * 3 * n, s));
    MD_CUDA_TRY(c, cudaMemsetAsync(B.U, 0, sizeof(double) * 3 * n, s));
    MD_CUDA_TRY(c, cudaMemsetAsync(B.acc, 0, sizeof(double) * nrep * NB, s));
    for (int sg = nseg - 1; sg >= 0; sg--) {
        const int m0 = sg * C, m1 = std::min(K, m0 + C);
        /* recompute the segment from its checkpoint, as the forward run did */
        launch_scatter_in(c, kp, 0, B.ck_x + 3 * (size_t)n * sg);
        launch_scatter_in(c, kp, 1, B.ck_v + 3 * (size_t)n * sg);
        launch_rebuild(c, kp, true, true);
        launch_forces(c, kp, true, MD_TERM_ALL);
        MD_CUDA_TRY(c, cudaMemcpyAsync(B.seg, B.ck_x + 3 * (size_t)n * sg, sizeof(double) * 3 * n,
                                       cudaMemcpyDeviceToDevice, s));
        for (int st = m0; st < m1; st++) {
            step(st);
            launch_gather_out(c, kp, 0, c->io_dev);
            MD_CUDA_TRY(c, cudaMemcpyAsync(B.seg + 3 * (size_t)n * (st + 1 - m0), c->io_dev,
                                           sizeof(double) * 3 * n, cudaMemcpyDeviceToDevice, s));
        }
        /* sweep the segment's frames backwards (its last frame belongs to
         * the later segment, except at the end of the trajectory) */
        for (int m = (m1 == K ? m1 : m1 - 1); m >= m0; m--) {
            launch_scatter_in(c, kp, 0, B.seg + 3 * (size_t)n * (m - m0));
            launch_check(c, kp);
            launch_rebuild(c, kp, false, false);
            ap.with_w = m < K ? 1 : 0;
            if (m < K)
                k_adj_w<<<agrid, 256, 0, s>>>(n, (double)c->dt, 1, m >= 1 ? 2.0 : 1.0, c->perm, c->kick,
                                               B.U, B.P, B.w4);
            launch_back(c, ap, B.rtab, B.w4, B.G, B.part);
            if (c->has_bonds || c->has_angles)
                k_adj_bonded<<<agrid, 256, 0, s>>>(n, c->pitch, ap, c->reps_dev, c->arep, c->pos4, B.w4, c->bl_s,
                                                    c->bl_sn, c->al_s, c->al_sn, c->bonded_par, c->has_bonds,
                                                    c->has_angles, B.G);
            k_adj_param<<<(nrep * NB * 32 + 255) / 256, 256, 0, s>>>(nrep, NB, c->reps_dev, B.part, B.acc);
            k_adj_acc<<<agrid, 256, 0, s>>>(n, c->pitch, c->perm, B.G, B.P);
        }
    }
    std::vector<double> acc((size_t)nrep * NB);
    MD_CUDA_TRY(c, cudaMemcpyAsync(acc.data(), B.acc, sizeof(double) * acc.size(), cudaMemcpyDeviceToHost, s));
    /* leave the context at the end of the trajectory */
    launch_scatter_in(c, kp, 0, B.xK);
    launch_scatter_in(c, kp, 1, B.vK);
    launch_rebuild(c, kp, true, true);
    launch_forces(c, kp, true, MD_TERM_ALL);
    launch_thermo_from_state(c, kp, 1);
    MD_CUDA_TRY(c, cudaStreamSynchronize(s));
    MD_CUDA_TRY(c, cudaGetLastError());
    for (int r = 0; r < nrep; r++) {
        const double *a = acc.data() + (size_t)r * NB;
        for (int k = 0; k < MD_MAXTYPE * MD_MAXTYPE; k++) {
            dlj1[(size_t)r * MD_MAXTYPE * MD_MAXTYPE + k] = 0.0;
            dlj2[(size_t)r * MD_MAXTYPE * MD_MAXTYPE + k] = 0.0;
        }
        for (int ti = 0; ti < nt; ti++)
            for (int tj = 0; tj < nt; tj++) {
                dlj1[(size_t)r * MD_MAXTYPE * MD_MAXTYPE + ti * MD_MAXTYPE + tj] = a[ti * 2 * nt + tj];
                dlj2[(size_t)r * MD_MAXTYPE * MD_MAXTYPE + ti * MD_MAXTYPE + tj] = a[ti * 2 * nt + nt + tj];
            }
        dlns[r] = a[NB - 1];
    }
    return MD_OK;
}
