/*
 * k_cells.cu -- neighbour-list maintenance: displacement check, cell binning,
 * Hilbert-order atom sort and the list build.
 *
 * Semantics follow neighborlist.cu: the list of atom i holds every j != i,
 * not excluded, with FP32 min-image r^2 < rskinsq evaluated exactly as the
 * reference writes it (neighborlist.cu:268-283; each operation rounded on its
 * own, so the set is bit-identical to the O(N^2) kernel's); it is rebuilt when
 * any atom moved >= skin/2 since the last build (neighborlist.cu:157-176).
 * Unlike the reference the candidates come from the 27..125 cells around i
 * (cells of side >= rl/2), the atoms are re-sorted along a Hilbert curve of
 * cells at every build, and the rebuild decision never leaves the device.
 */
#include <algorithm>
#include <type_traits>

#include "md_device.cuh"

namespace {

__global__ void k_check(md_kparams kp, const float4 *__restrict__ pos4,
                        const float4 *__restrict__ pos_old, md_devstate *st)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= kp.n) return;
    if (md_rsq_exact(pos4[i], pos_old[i], kp) >= kp.rmaxdif) st->update = 1;
}

/* Cell rank (Hilbert order) of atom i and its count in the cell. */
__device__ __forceinline__ void key_one(const md_kparams &kp, int i, const float4 *__restrict__ pos4,
                                        const int *__restrict__ cell_rank, int *key, int *cell_count)
{
    float4 p = pos4[i];
    int cx = cell_of(cell_coord(p.x, kp.box[0], kp.boxi[0], kp.centered), kp.box[0], kp.binlen[0], kp.ncell[0]);
    int cy = cell_of(cell_coord(p.y, kp.box[1], kp.boxi[1], kp.centered), kp.box[1], kp.binlen[1], kp.ncell[1]);
    int cz = cell_of(cell_coord(p.z, kp.box[2], kp.boxi[2], kp.centered), kp.box[2], kp.binlen[2], kp.ncell[2]);
    int r = cell_rank[cx + kp.ncell[0] * (cy + kp.ncell[1] * cz)];
    key[i] = r;
    atomicAdd(&cell_count[r], 1);
}

/* Cell rank (Hilbert order) of every atom and the per-cell counts. */
__global__ void k_cell_key(md_kparams kp, const md_devstate *st, int always,
                           const float4 *__restrict__ pos4, const int *__restrict__ cell_rank,
                           int *key, int *cell_count)
{
    pdl_wait();      /* launched after the previous pass (programmatic launch) */
    pdl_trigger();
    if (!always && !st->update) return;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= kp.n) return;
    key_one(kp, i, pos4, cell_rank, key, cell_count);
}

/* The same for a batch: each atom is tested with its replica's box and skin. */
__global__ void k_check_b(int n, const md_rep *__restrict__ reps, const int *__restrict__ arep,
                          const float4 *__restrict__ pos4, const float4 *__restrict__ pos_old,
                          md_devstate *st, int *rep_upd)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int r = arep[i];
    const md_rep &R = reps[r];
    if (md_rsq_box(pos4[i], pos_old[i], R.box, R.boxi) >= R.rmaxdif) {
        st->update = 1;
        rep_upd[r] = 1;
    }
}

/* Cell keys of a batch: the replica's cell grid, ranks offset by its first
 * cell, so every replica's cells (and atoms) stay one contiguous range.
 * Only replicas with a rebuild request are re-binned; every other replica
 * keeps its order, cell ranges and list rows untouched by all build passes. */
__global__ void k_cell_key_b(int n, int centered, const md_rep *__restrict__ reps,
                             const int *__restrict__ arep,
                             const md_devstate *st, int always, const int *__restrict__ rep_upd,
                             const float4 *__restrict__ pos4, const int *__restrict__ cell_rank,
                             int *key, int *cell_count)
{
    if (!always && !st->update) return;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int rep = arep[i];
    if (!rep_upd[rep]) return;
    const md_rep &R = reps[rep];
    float4 p = pos4[i];
    int cx = cell_of(cell_coord(p.x, R.box[0], R.boxi[0], centered), R.box[0], R.binlen[0], R.ncell[0]);
    int cy = cell_of(cell_coord(p.y, R.box[1], R.boxi[1], centered), R.box[1], R.binlen[1], R.ncell[1]);
    int cz = cell_of(cell_coord(p.z, R.box[2], R.boxi[2], centered), R.box[2], R.binlen[2], R.ncell[2]);
    int r = cell_rank[R.cell0 + cx + R.ncell[0] * (cy + R.ncell[1] * cz)];
    key[i] = r;
    atomicAdd(&cell_count[r], 1);
}

/* Per-replica exclusive scan of the cell counts, one warp per replica being
 * rebuilt: its cells start at its first atom.  Counters are zeroed for the
 * next build. */
__global__ void k_cell_scan_b(const md_devstate *st, int always, int nrep,
                              const md_rep *__restrict__ reps, const int *__restrict__ rep_upd,
                              int *cell_count, int *cell_start, int *cell_fill)
{
    if (!always && !st->update) return;
    const int r = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (r >= nrep || !rep_upd[r]) return;
    const md_rep &R = reps[r];
    int run = R.atom0;
    for (int k0 = 0; k0 < R.ncells; k0 += 32) {
        const int k = k0 + lane;
        const int c = R.cell0 + k;
        int cnt = k < R.ncells ? cell_count[c] : 0;
        int incl = cnt;
        for (int o = 1; o < 32; o <<= 1) {
            int v = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += v;
        }
        if (k < R.ncells) {
            cell_start[c] = run + incl - cnt;
            cell_count[c] = 0;
            cell_fill[c] = 0;
        }
        run += __shfl_sync(0xffffffffu, incl, 31);
    }
    if (lane == 0) cell_start[R.cell0 + R.ncells] = run;   /* = the next replica's first atom */
}

/* Rebuild every replica of a batch (forced builds). */
__global__ void k_flag_all(int *rep_upd, int nrep)
{
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r < nrep) rep_upd[r] = 1;
}

/* Ends a rebuild of a batch: counts the build and the rebuilt replicas'
 * builds and clears the requests. */
__global__ void k_clear_update_b(md_devstate *st, int always, int *rep_upd, md_repstate *repst,
                                 int nrep)
{
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r == 0) {
        if (always || st->update) st->builds += 1;
        st->update = 0;
        st->cell_next = 0;
    }
    if (r < nrep && rep_upd[r]) {
        repst[r].builds += 1;
        rep_upd[r] = 0;
    }
}

/* Exclusive scan of the cell counts by one block of NT threads, then (ZERO)
 * zero the counters for the next build; returns the total in thread 0.
 * Without ZERO, cell_start may be cell_count itself (each round loads its
 * counts before it writes their starts).  In
 * rounds of NT x SCAN_K cells: the counts pass through shared memory, so
 * that global loads and stores are coalesced (one SM issues them all) while
 * each thread scans SCAN_K consecutive counts; warps scan their threads'
 * sums with shuffles and warp 0 the warp totals.  Shared index i is stored
 * at i + i / SCAN_K, so the per-thread reads hit distinct banks. */
constexpr int SCAN_K = 8;
__device__ __forceinline__ int scan_pad(int i) { return i + i / SCAN_K; }

template <int NT, bool ZERO = true>
__device__ __forceinline__ int scan_cells(int ncells, int *cell_count, int *cell_start, int *cell_fill)
{
    constexpr int N = NT * SCAN_K;
    __shared__ int buf[N + N / SCAN_K];
    __shared__ int wsum[32];
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    int carry = 0;
    for (int base = 0; base < ncells; base += N) {
#pragma unroll
        for (int k = 0; k < SCAN_K; k++) {
            const int i = k * NT + t, g = base + i;
            buf[scan_pad(i)] = g < ncells ? cell_count[g] : 0;
        }
        __syncthreads();
        int v[SCAN_K], s = 0;
#pragma unroll
        for (int k = 0; k < SCAN_K; k++) {
            v[k] = buf[scan_pad(t * SCAN_K + k)];
            s += v[k];
        }
        int incl = s;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += y;
        }
        if (lane == 31) wsum[w] = incl;
        __syncthreads();
        if (w == 0) {
            int x = lane < NT / 32 ? wsum[lane] : 0;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int y = __shfl_up_sync(0xffffffffu, x, o);
                if (lane >= o) x += y;
            }
            wsum[lane] = x;   /* inclusive over warps */
        }
        __syncthreads();
        int run = carry + (w > 0 ? wsum[w - 1] : 0) + incl - s;
#pragma unroll
        for (int k = 0; k < SCAN_K; k++) {
            buf[scan_pad(t * SCAN_K + k)] = run;
            run += v[k];
        }
        carry += wsum[NT / 32 - 1];
        __syncthreads();
#pragma unroll
        for (int k = 0; k < SCAN_K; k++) {
            const int i = k * NT + t, g = base + i;
            if (g < ncells) {
                cell_start[g] = buf[scan_pad(i)];
                if (ZERO) {
                    cell_count[g] = 0;
                    cell_fill[g] = 0;
                }
            }
        }
        __syncthreads();   /* buf and wsum are rewritten by the next round */
    }
    return carry;
}

/* The scan as its own pass (one block of 1024 threads); cell_start has
 * ncells + 1 entries. */
__global__ void __launch_bounds__(1024) k_cell_scan(md_kparams kp, md_devstate *st, int always,
                                                    int ncells, int *cell_count, int *cell_start,
                                                    int *cell_fill)
{
    pdl_wait();      /* launched after the previous pass (programmatic launch) */
    pdl_trigger();
    if (!always && !st->update) return;
    const int total = scan_cells<1024>(ncells, cell_count, cell_start, cell_fill);
    if (threadIdx.x == 0) {
        cell_start[ncells] = total;
        st->builds += 1;
    }
}

/* In a batch (arep, rep_upd non-null) the passes below touch only the atoms
 * and cells of replicas being rebuilt. */
__global__ void k_cell_scatter(md_kparams kp, const md_devstate *st, int always,
                               const int *__restrict__ key, const int *__restrict__ cell_start,
                               int *cell_fill, int *src, const int *__restrict__ arep,
                               const int *__restrict__ rep_upd)
{
    pdl_wait();      /* launched after the previous pass (programmatic launch) */
    pdl_trigger();
    if (!always && !st->update) return;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= kp.n) return;
    if (arep && !rep_upd[arep[i]]) return;
    int r = key[i];
    src[cell_start[r] + atomicAdd(&cell_fill[r], 1)] = i;
}

/* Within each cell, order atoms by original index: the sorted order is then a
 * function of the positions alone.  One warp per cell: each atom's place is
 * the number of the cell's atoms with a smaller original index (indices are
 * distinct), counted with shuffles; cells of more than 4 x 32 atoms (far
 * denser than any liquid at these cell sizes) are sorted by one lane. */
constexpr int ORD_MAX = 4;
/* The rank sort of one cell's atoms (one warp). */
__device__ __forceinline__ void order_cell(int c, const int *__restrict__ cell_start,
                                           const int *__restrict__ perm, int *src,
                                           const int *__restrict__ crep,
                                           const int *__restrict__ rep_upd, int lane)
{
    if (crep && !rep_upd[crep[c]]) return;
    const int b = cell_start[c], n = cell_start[c + 1] - b;
    if (n <= 1) return;
    if (n <= 32 * ORD_MAX) {
        int a[ORD_MAX], key[ORD_MAX], rank[ORD_MAX];
#pragma unroll
        for (int q = 0; q < ORD_MAX; q++) {
            const int k = q * 32 + lane;
            a[q] = k < n ? src[b + k] : 0;
            key[q] = k < n ? perm[a[q]] : 0x7fffffff;
            rank[q] = 0;
        }
#pragma unroll
        for (int q2 = 0; q2 < ORD_MAX; q2++) {
            if (q2 * 32 >= n) break;
            const int m = min(32, n - q2 * 32);
            for (int j = 0; j < m; j++) {
                const int kj = __shfl_sync(0xffffffffu, key[q2], j);
#pragma unroll
                for (int q = 0; q < ORD_MAX; q++) rank[q] += kj < key[q] ? 1 : 0;
            }
        }
        __syncwarp();   /* every read of src above precedes the writes below */
#pragma unroll
        for (int q = 0; q < ORD_MAX; q++)
            if (q * 32 + lane < n) src[b + rank[q]] = a[q];
        return;
    }
    if (lane != 0) return;
    for (int k = b + 1; k < b + n; k++) {
        int a = src[k], ka = perm[a];
        int m = k - 1;
        while (m >= b && perm[src[m]] > ka) {
            src[m + 1] = src[m];
            m--;
        }
        src[m + 1] = a;
    }
}

__global__ void k_cell_order(md_kparams kp, const md_devstate *st, int always, int ncells,
                             const int *__restrict__ cell_start, const int *__restrict__ perm,
                             int *src, const int *__restrict__ crep, const int *__restrict__ rep_upd)
{
    pdl_wait();      /* launched after the previous pass (programmatic launch) */
    pdl_trigger();
    if (!always && !st->update) return;
    const int lane = threadIdx.x & 31, nw = (int)((gridDim.x * blockDim.x) >> 5);
    for (int c = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5); c < ncells; c += nw) {
        order_cell(c, cell_start, perm, src, crep, rep_upd, lane);
        __syncwarp();
    }
}

/* Sorted slot s takes the state of atom src[s] (into the staging arrays). */
__device__ __forceinline__ void permute_one(const md_kparams &kp, int s, const int *__restrict__ src,
                                            const double *__restrict__ x, const double *__restrict__ v,
                                            const double *__restrict__ mass, const double *__restrict__ kick,
                                            const float4 *__restrict__ pos4, const int *__restrict__ perm,
                                            const int *__restrict__ type, double *tmp_d, float4 *tmp4,
                                            int *tmp_i)
{
    int o = src[s], P = kp.pitch;
    for (int d = 0; d < 3; d++) {
        tmp_d[d * P + s] = x[d * P + o];
        tmp_d[(3 + d) * P + s] = v[d * P + o];
    }
    tmp_d[6 * P + s] = mass[o];
    tmp_d[7 * P + s] = kick[o];
    tmp4[s] = pos4[o];
    tmp_i[s] = perm[o];
    tmp_i[P + s] = type[o];
}

/* The staged state back into the per-atom arrays, and the inverse order. */
__device__ __forceinline__ void copyback_one(const md_kparams &kp, int s, const double *__restrict__ tmp_d,
                                             const float4 *__restrict__ tmp4, const int *__restrict__ tmp_i,
                                             double *x, double *v, double *mass, double *kick, float4 *pos4,
                                             int *perm, int *iperm, int *type)
{
    int P = kp.pitch;
    for (int d = 0; d < 3; d++) {
        x[d * P + s] = tmp_d[d * P + s];
        v[d * P + s] = tmp_d[(3 + d) * P + s];
    }
    mass[s] = tmp_d[6 * P + s];
    kick[s] = tmp_d[7 * P + s];
    pos4[s] = tmp4[s];
    int o = tmp_i[s];
    perm[s] = o;
    iperm[o] = s;
    type[s] = tmp_i[P + s];
}

/* Exclusions and bonded lists of sorted slot s in the new sorted indices. */
__device__ __forceinline__ void remap_one(const md_kparams &kp, int s, const int *__restrict__ perm,
                                          const int *__restrict__ iperm, const uint4 *__restrict__ excl_orig,
                                          uint4 *excl_s, const int2 *__restrict__ bl_o,
                                          const int *__restrict__ bl_on, int2 *bl_s, int *bl_sn,
                                          const int4 *__restrict__ al_o, const int *__restrict__ al_on,
                                          int4 *al_s, int *al_sn, int has_bonds, int has_angles)
{
    int o = perm[s], P = kp.pitch;
    uint4 e = excl_orig[o];
    uint4 m;
    m.x = e.x == MD_EXCL_NONE ? MD_EXCL_NONE : (unsigned)iperm[e.x];
    m.y = e.y == MD_EXCL_NONE ? MD_EXCL_NONE : (unsigned)iperm[e.y];
    m.z = e.z == MD_EXCL_NONE ? MD_EXCL_NONE : (unsigned)iperm[e.z];
    m.w = e.w == MD_EXCL_NONE ? MD_EXCL_NONE : (unsigned)iperm[e.w];
    excl_s[s] = m;
    if (has_bonds) {
        int nb = bl_on[o];
        for (int k = 0; k < nb; k++) {
            int2 b = bl_o[4 * o + k];
            bl_s[k * P + s] = make_int2(iperm[b.x], b.y);
        }
        bl_sn[s] = nb;
    }
    if (has_angles) {
        int na = al_on[o];
        for (int k = 0; k < na; k++) {
            int4 a = al_o[4 * o + k];
            al_s[k * P + s] = make_int4(a.x, iperm[a.y], iperm[a.z], a.w);
        }
        al_sn[s] = na;
    }
}

__global__ void k_permute(md_kparams kp, const md_devstate *st, int always,
                          const int *__restrict__ src, const double *__restrict__ x,
                          const double *__restrict__ v, const double *__restrict__ mass,
                          const double *__restrict__ kick,
                          const float4 *__restrict__ pos4, const int *__restrict__ perm,
                          const int *__restrict__ type, double *tmp_d, float4 *tmp4, int *tmp_i,
                          const int *__restrict__ arep, const int *__restrict__ rep_upd)
{
    pdl_wait();      /* launched after the previous pass (programmatic launch) */
    pdl_trigger();
    if (!always && !st->update) return;
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= kp.n) return;
    if (arep && !rep_upd[arep[s]]) return;   /* atoms stay inside their replica's range */
    permute_one(kp, s, src, x, v, mass, kick, pos4, perm, type, tmp_d, tmp4, tmp_i);
}

__global__ void k_copyback(md_kparams kp, const md_devstate *st, int always,
                           const double *__restrict__ tmp_d, const float4 *__restrict__ tmp4,
                           const int *__restrict__ tmp_i, double *x, double *v, double *mass,
                           double *kick, float4 *pos4, int *perm, int *iperm, int *type,
                           const int *__restrict__ arep, const int *__restrict__ rep_upd)
{
    pdl_wait();      /* launched after the previous pass (programmatic launch) */
    pdl_trigger();
    if (!always && !st->update) return;
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= kp.n) return;
    if (arep && !rep_upd[arep[s]]) return;
    copyback_one(kp, s, tmp_d, tmp4, tmp_i, x, v, mass, kick, pos4, perm, iperm, type);
}

/* Exclusions and bonded lists re-expressed in the new sorted indices. */
__global__ void k_remap(md_kparams kp, const md_devstate *st, int always,
                        const int *__restrict__ perm, const int *__restrict__ iperm,
                        const uint4 *__restrict__ excl_orig, uint4 *excl_s,
                        const int2 *__restrict__ bl_o, const int *__restrict__ bl_on, int2 *bl_s,
                        int *bl_sn, const int4 *__restrict__ al_o, const int *__restrict__ al_on,
                        int4 *al_s, int *al_sn, int has_bonds, int has_angles)
{
    pdl_wait();      /* launched after the previous pass (programmatic launch) */
    pdl_trigger();
    if (!always && !st->update) return;
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= kp.n) return;
    remap_one(kp, s, perm, iperm, excl_orig, excl_s, bl_o, bl_on, bl_s, bl_sn, al_o, al_on, al_s, al_sn,
              has_bonds, has_angles);
}

/* Ends a rebuild (or a step without one): the next step's check sets the
 * request again. */
__global__ void k_clear_update(md_devstate *st)
{
    pdl_wait();
    st->update = 0;
    st->cell_next = 0;
}

/* First node of a captured step graph: the rebuild condition of its first
 * step comes from the check done by the step before the graph. */
__global__ void k_set_condition(cudaGraphConditionalHandle h, const md_devstate *st)
{
    cudaGraphSetConditional(h, st->update ? 1u : 0u);
}

/* List build: TPA lanes per atom scan the stencil cells; lane l tests the
 * candidates l, l+TPA, ... of each cell and the lanes append their hits in
 * candidate order with a ballot, so the list order is fixed by the cell
 * traversal order alone. */
template <int TPA>
__global__ void __launch_bounds__(256) k_build_list(
    md_kparams kp, md_devstate *st, int always, const float4 *__restrict__ pos4,
    const int *__restrict__ type, const uint4 *__restrict__ excl_s,
    const int *__restrict__ cell_rank, const int *__restrict__ cell_start,
    const unsigned *__restrict__ type_mask, unsigned *nl, int *nl_n, float4 *pos_old)
{
    pdl_wait();      /* launched after the previous pass (programmatic launch) */
    pdl_trigger();
    if (!always && !st->update) return;
    int gt = blockIdx.x * blockDim.x + threadIdx.x;
    int i = gt / TPA, lane = gt % TPA;
    int lane_w = threadIdx.x & 31;
    unsigned gmask = (TPA == 32) ? 0xffffffffu : (((1u << TPA) - 1u) << (lane_w & ~(TPA - 1)));
    bool active = i < kp.n;
    int ii = active ? i : 0;
    float4 p = pos4[ii];
    int ti = type[ii];
    uint4 ex = excl_s[ii];
    unsigned tmask = type_mask[ti];
    int c3[3];
    for (int d = 0; d < 3; d++)
        c3[d] = cell_of(cell_coord(d == 0 ? p.x : (d == 1 ? p.y : p.z), kp.box[d], kp.boxi[d], kp.centered),
                        kp.box[d], kp.binlen[d], kp.ncell[d]);
    int lo[3], hi[3];
    for (int d = 0; d < 3; d++) {
        if (kp.stencil[d] < 0) { lo[d] = 0; hi[d] = kp.ncell[d] - 1; }
        else { lo[d] = c3[d] - kp.stencil[d]; hi[d] = c3[d] + kp.stencil[d]; }
    }
    int cnt = 0;
    for (int zz = lo[2]; zz <= hi[2]; zz++) {
        int cz = zz < 0 ? zz + kp.ncell[2] : (zz >= kp.ncell[2] ? zz - kp.ncell[2] : zz);
        for (int yy = lo[1]; yy <= hi[1]; yy++) {
            int cy = yy < 0 ? yy + kp.ncell[1] : (yy >= kp.ncell[1] ? yy - kp.ncell[1] : yy);
            for (int xx = lo[0]; xx <= hi[0]; xx++) {
                int cx = xx < 0 ? xx + kp.ncell[0] : (xx >= kp.ncell[0] ? xx - kp.ncell[0] : xx);
                int r = cell_rank[cx + kp.ncell[0] * (cy + kp.ncell[1] * cz)];
                int b = cell_start[r], e = cell_start[r + 1];
                for (int j0 = b; j0 < e; j0 += TPA) {
                    int j = j0 + lane;
                    bool ok = false;
                    unsigned entry = 0;
                    if (active && j < e) {
                        float4 q = pos4[j];
                        unsigned uj = (unsigned)j;
                        int tj = type[j];
                        ok = md_rsq_exact(p, q, kp) < kp.rskinsq && j != i && uj != ex.x &&
                             uj != ex.y && uj != ex.z && uj != ex.w && !((tmask >> tj) & 1u);
                        entry = uj | ((unsigned)tj << MD_TYPE_SHIFT);
                    }
                    unsigned bal = __ballot_sync(gmask, ok);
                    if (ok) {
                        int slot = cnt + __popc(bal & ((1u << lane_w) - 1u));
                        if (slot < kp.cap) nl[(size_t)i * kp.cap + slot] = entry;
                    }
                    cnt += __popc(bal);
                }
            }
        }
    }
    if (active) {
        /* pad the row to the next multiple of 32 with the atom itself */
        int lim = min(kp.cap, (cnt + MD_LIST_QUANTUM - 1) / MD_LIST_QUANTUM * MD_LIST_QUANTUM);
        unsigned self = (unsigned)i | ((unsigned)ti << MD_TYPE_SHIFT);
        for (int k = cnt + lane; k < lim; k += TPA) nl[(size_t)i * kp.cap + k] = self;
    }
    if (active && lane == 0) {
        nl_n[i] = cnt < kp.cap ? cnt : kp.cap;
        pos_old[i] = p;
        if (cnt > kp.cap) atomicMax(&st->list_overflow, cnt);
    }
}

/* List build, one warp per cell: every atom of a cell shares the cell's
 * stencil.  The warp first gathers the stencil cells' atom ranges into
 * shared memory (in traversal order) with their prefix sums, then streams the
 * concatenated candidates 32 at a time (lane = candidate, its stencil cell
 * found by stepping forward through the prefix sums).  A conservative test
 * against the bounding box of the cell's atoms drops the candidates (about a
 * third) that no atom of the cell can reach; the rest enter a per-warp queue
 * in candidate order, and each full queue of 32 is tested exactly against
 * the cell's atoms, two at a time, a ballot per atom appending the hits to
 * its list.  Entries land in the
 * same order as in k_build_list (stencil cells in traversal order, ascending
 * j), so both builders produce identical lists. */
constexpr int CW_WARPS = 8;   /* warps per block (fewer blocks: fewer grid-barrier arrivals) */
constexpr int CW_MAXI = 32;
constexpr int CW_MAXST = 128;

/* Cell geometry seen by one warp: the system's, or in a batch the replica's
 * that owns the cell. */
struct cell_geom {
    float L[3], Li[3], rskinsq;
    int nc[3], sten[3], shift, lin0;
};

/* The list rows of the atoms of cell r (sorted rank), built by one warp. */
template <bool BATCH>
__device__ __forceinline__ void build_cell(
    int r, const md_kparams &kp, md_devstate *st, const float4 *__restrict__ pos4,
    const int *__restrict__ type, const uint4 *__restrict__ excl_s,
    const int *__restrict__ cell_rank, const int *__restrict__ cell_lin,
    const int *__restrict__ cell_start, const unsigned *__restrict__ type_mask, unsigned *nl,
    int *nl_n, float4 *pos_old, const md_rep *__restrict__ reps, const int *__restrict__ crep,
    const int *__restrict__ rep_upd)
{
    __shared__ float4 s_p[CW_WARPS][CW_MAXI];
    /* the group's coordinates once more by axis, so that two atoms' x (y, z)
     * are one aligned 8-byte load; slots past the group hold a far point */
    __shared__ __align__(16) float s_h[CW_WARPS][3][CW_MAXI];
    __shared__ uint4 s_ex[CW_WARPS][CW_MAXI];
    __shared__ unsigned s_tm[CW_WARPS][CW_MAXI];
    __shared__ int s_jb[CW_WARPS][CW_MAXST];
    __shared__ int s_pre[CW_WARPS][CW_MAXST + 1];
    __shared__ unsigned char s_sh[CW_WARPS][CW_MAXST];   /* image code per stencil cell */
    __shared__ float4 s_fq[CW_WARPS][64];                 /* queue of near candidates: position, */
    __shared__ unsigned s_fe[CW_WARPS][64];               /* list entry (j | type << 29) */
    __shared__ unsigned char s_fc[CW_WARPS][64];          /* and image code */
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int ib = cell_start[r], ie = cell_start[r + 1];
    if (ib == ie) return;
    cell_geom G;
    if (BATCH) {
        const int rr = crep[r];
        if (!rep_upd[rr]) return;   /* this replica keeps its list */
        const md_rep &R = reps[rr];
        for (int d = 0; d < 3; d++) {
            G.L[d] = R.box[d]; G.Li[d] = R.boxi[d]; G.nc[d] = R.ncell[d]; G.sten[d] = R.stencil[d];
        }
        G.rskinsq = R.rskinsq; G.shift = R.cell_shift && kp.centered; G.lin0 = R.cell0;
    } else {
        for (int d = 0; d < 3; d++) {
            G.L[d] = kp.box[d]; G.Li[d] = kp.boxi[d]; G.nc[d] = kp.ncell[d]; G.sten[d] = kp.stencil[d];
        }
        G.rskinsq = kp.rskinsq; G.shift = kp.cell_shift; G.lin0 = 0;
    }
    const int lin = cell_lin[r];
    const int nx = G.nc[0], ny = G.nc[1], nz = G.nc[2];
    const int c3[3] = {lin % nx, (lin / nx) % ny, lin / (nx * ny)};
    int lo[3], len[3];
    for (int d = 0; d < 3; d++) {
        if (G.sten[d] < 0) { lo[d] = 0; len[d] = G.nc[d]; }
        else { lo[d] = c3[d] - G.sten[d]; len[d] = 2 * G.sten[d] + 1; }
    }
    const int nst = len[0] * len[1] * len[2];   /* <= 125 with cells of side >= rl/2 */
    /* stencil ranges in traversal order (z outer, x inner); lane k takes k, k+32, ... */
    int run = 0;
    for (int k0 = 0; k0 < nst; k0 += 32) {
        int k = k0 + lane;
        int cnt = 0, jb = 0, code = 0;
        if (k < nst) {
            int dx = k % len[0], dy = (k / len[0]) % len[1], dz = k / (len[0] * len[1]);
            int xx = lo[0] + dx, yy = lo[1] + dy, zz = lo[2] + dz;
            /* code per axis: 0 no image, 1 the cell wrapped from below (the
             * reference's rint(d/L) = -1), 2 from above (+1) */
            code = (xx < 0 ? 1 : (xx >= nx ? 2 : 0)) | ((yy < 0 ? 1 : (yy >= ny ? 2 : 0)) << 2) |
                   ((zz < 0 ? 1 : (zz >= nz ? 2 : 0)) << 4);
            int cx = xx < 0 ? xx + nx : (xx >= nx ? xx - nx : xx);
            int cy = yy < 0 ? yy + ny : (yy >= ny ? yy - ny : yy);
            int cz = zz < 0 ? zz + nz : (zz >= nz ? zz - nz : zz);
            int r2 = cell_rank[G.lin0 + cx + nx * (cy + ny * cz)];
            jb = cell_start[r2];
            cnt = cell_start[r2 + 1] - jb;
        }
        int incl = cnt;
        for (int o = 1; o < 32; o <<= 1) {
            int v = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += v;
        }
        if (k < nst) {
            s_jb[w][k] = jb;
            s_pre[w][k] = run + incl - cnt;
            s_sh[w][k] = (unsigned char)code;
        }
        run += __shfl_sync(0xffffffffu, incl, 31);
    }
    if (lane == 0) s_pre[w][nst] = run;
    const int total = run;
    const unsigned lt = (1u << lane) - 1u;
    const float L0 = G.L[0], L1 = G.L[1], L2 = G.L[2];
    __syncwarp();
    for (int i0 = ib; i0 < ie; i0 += CW_MAXI) {
        const int ni = min(CW_MAXI, ie - i0);
        bool any_excl = false;
        {
            const float4 p = lane < ni ? pos4[i0 + lane] : make_float4(1e30f, 1e30f, 1e30f, 0.0f);
            s_h[w][0][lane] = p.x;
            s_h[w][1][lane] = p.y;
            s_h[w][2][lane] = p.z;
        }
        if (lane < ni) {
            int i = i0 + lane;
            s_p[w][lane] = pos4[i];
            uint4 ex = excl_s[i];
            s_ex[w][lane] = ex;
            unsigned tm = type_mask[type[i]];
            s_tm[w][lane] = tm;
            any_excl = ex.x != MD_EXCL_NONE || ex.y != MD_EXCL_NONE || ex.z != MD_EXCL_NONE ||
                       ex.w != MD_EXCL_NONE || tm != 0u;
        }
        const unsigned excl_bits = __ballot_sync(0xffffffffu, any_excl);
        __syncwarp();
        int mycnt = 0;   /* list length of atom i0 + lane */
        /* The exact test of 32 queued candidates against every atom of the
         * group; a ballot appends the hits to each atom's row in candidate
         * order.  An atom's row offset changes only in its own iteration, so
         * each iteration takes it from the counts at the start of the batch
         * and the iterations are independent (unrolled by 4: 156 against 168
         * us per build of 64000 ions with the count as a loop-carried
         * register). */
        auto process = [&](int cnt) {
            const bool vj = lane < cnt;
            const float4 q = vj ? s_fq[w][lane] : make_float4(0.f, 0.f, 0.f, 0.f);
            const unsigned entry = vj ? s_fe[w][lane] : 0u;
            const int code = vj ? s_fc[w][lane] : 0;
            const unsigned uj = entry & MD_INDEX_MASK;
            const int tj = (int)(entry >> MD_TYPE_SHIFT);
            /* exact images: u = L * rint(d / L) is -L, 0 or +L by stencil cell */
            const float ux = (code & 3) == 1 ? -L0 : ((code & 3) == 2 ? L0 : 0.0f);
            const float uy = ((code >> 2) & 3) == 1 ? -L1 : (((code >> 2) & 3) == 2 ? L1 : 0.0f);
            const float uz = ((code >> 4) & 3) == 1 ? -L2 : (((code >> 4) & 3) == 2 ? L2 : 0.0f);
            /* the group member this candidate is, if any (never its own neighbour) */
            const int selfa = (vj && (int)uj >= i0 && (int)uj < i0 + ni) ? (int)uj - i0 : -1;
            /* two copies of the loop: with and without the exclusion tests */
            auto loop = [&](auto with_excl) {
                unsigned *rowp = nl + (size_t)i0 * kp.cap;
                const int cnt0 = mycnt;
                int inc = 0;
#pragma unroll 4
                for (int a = 0; a < ni; a++, rowp += kp.cap) {
                    const float4 p = s_p[w][a];
                    float rsq;
                    if (G.shift) {
                        /* fl(fl(px - qx) - u) is the reference's fl(d - fl(L rint(d/L))) */
                        float dx = __fsub_rn(__fsub_rn(p.x, q.x), ux);
                        float dy = __fsub_rn(__fsub_rn(p.y, q.y), uy);
                        float dz = __fsub_rn(__fsub_rn(p.z, q.z), uz);
                        rsq = __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
                    } else {
                        rsq = md_rsq_box(p, q, G.L, G.Li);
                    }
                    bool ok = vj && rsq < G.rskinsq && a != selfa;
                    if (decltype(with_excl)::value && ((excl_bits >> a) & 1u)) {
                        uint4 ex = s_ex[w][a];
                        ok = ok && uj != ex.x && uj != ex.y && uj != ex.z && uj != ex.w &&
                             !((s_tm[w][a] >> tj) & 1u);
                    }
                    const unsigned bal = __ballot_sync(0xffffffffu, ok);
                    const int base = __shfl_sync(0xffffffffu, cnt0, a);
                    if (ok) {
                        const int slot = base + __popc(bal & lt);
                        if (slot < kp.cap) rowp[slot] = entry;
                    }
                    if (lane == a) inc += __popc(bal);
                }
                mycnt = cnt0 + inc;
            };
            if (excl_bits) {
                loop(std::true_type());
            } else if (G.shift) {
                /* two group atoms per iteration: the differences and squares
                 * in packed f32x2 instructions, the two sums in scalar adds
                 * with explicit rounding (a packed multiply followed by a
                 * packed add may be contracted into a packed FMA by the code
                 * generator, which would change the rounding of r^2) */
                typedef v2<true> V;
                const V QX = V::make(q.x, q.x), QY = V::make(q.y, q.y), QZ = V::make(q.z, q.z);
                const V UX = V::make(ux, ux), UY = V::make(uy, uy), UZ = V::make(uz, uz);
                const float far = vj ? G.rskinsq : -1.0f;   /* no hit in an empty slot */
                const int cnt0 = mycnt;
                int inc = 0;
#pragma unroll 4
                for (int a = 0; a < ni; a += 2) {
                    const float2 hx = *reinterpret_cast<const float2 *>(&s_h[w][0][a]);
                    const float2 hy = *reinterpret_cast<const float2 *>(&s_h[w][1][a]);
                    const float2 hz = *reinterpret_cast<const float2 *>(&s_h[w][2][a]);
                    const V dx = (V::make(hx.x, hx.y) - QX) - UX;
                    const V dy = (V::make(hy.x, hy.y) - QY) - UY;
                    const V dz = (V::make(hz.x, hz.y) - QZ) - UZ;
                    float x0, x1, y0, y1, z0, z1;
                    (dx * dx).get(x0, x1);
                    (dy * dy).get(y0, y1);
                    (dz * dz).get(z0, z1);
                    const float r0 = __fadd_rn(__fadd_rn(x0, y0), z0);
                    const float r1 = __fadd_rn(__fadd_rn(x1, y1), z1);
#pragma unroll
                    for (int h = 0; h < 2; h++) {
                        const bool ok = (h ? r1 : r0) < far && a + h != selfa;
                        const unsigned bal = __ballot_sync(0xffffffffu, ok);
                        const int base = __shfl_sync(0xffffffffu, cnt0, a + h);
                        const int slot = base + __popc(bal & lt);
                        if (ok && slot < kp.cap) nl[(size_t)(i0 + a + h) * kp.cap + slot] = entry;
                        inc += lane == a + h ? __popc(bal) : 0;
                    }
                }
                mycnt = cnt0 + inc;
            } else {
                loop(std::false_type());
            }
        };
        /* Bounding box of the group: candidates farther than rl from it
         * cannot pass the exact test for any member and are dropped before
         * it (a conservative FP32 test; the exact test decides the rest). */
        float bx0 = 3.4e38f, by0 = 3.4e38f, bz0 = 3.4e38f, bx1 = -3.4e38f, by1 = -3.4e38f, bz1 = -3.4e38f;
        if (lane < ni) {
            const float4 p = s_p[w][lane];
            bx0 = bx1 = p.x;
            by0 = by1 = p.y;
            bz0 = bz1 = p.z;
        }
        for (int o = 16; o > 0; o >>= 1) {
            bx0 = fminf(bx0, __shfl_xor_sync(0xffffffffu, bx0, o));
            by0 = fminf(by0, __shfl_xor_sync(0xffffffffu, by0, o));
            bz0 = fminf(bz0, __shfl_xor_sync(0xffffffffu, bz0, o));
            bx1 = fmaxf(bx1, __shfl_xor_sync(0xffffffffu, bx1, o));
            by1 = fmaxf(by1, __shfl_xor_sync(0xffffffffu, by1, o));
            bz1 = fmaxf(bz1, __shfl_xor_sync(0xffffffffu, bz1, o));
        }
        const float near_sq = G.rskinsq * 1.001f + 1e-4f;
        int fill = 0;   /* queued candidates (in candidate order) */
        int kc = 0;     /* this lane's stencil cell: the largest k with s_pre[k] <= g */
        /* software pipelined: the next round's candidate (its stencil cell,
         * position and type) is located and loaded while this round's are
         * filtered (144 against 156 us per build of 64000 ions) */
        int jn = 0, cn = 0, tn = 0;
        bool vn = lane < total;
        float4 qn = make_float4(0.f, 0.f, 0.f, 0.f);
        if (vn) {
            while (s_pre[w][kc + 1] <= lane) kc++;
            jn = s_jb[w][kc] + (lane - s_pre[w][kc]);
            cn = s_sh[w][kc];
            qn = pos4[jn];
            tn = type[jn];
        }
        for (int g0 = 0; g0 < total; g0 += 32) {
            const int j = jn, code = cn, tj = tn;
            const bool vj = vn;
            const float4 q = qn;
            {
                const int g = g0 + 32 + lane;
                vn = g < total;
                if (vn) {
                    while (s_pre[w][kc + 1] <= g) kc++;
                    jn = s_jb[w][kc] + (g - s_pre[w][kc]);
                    cn = s_sh[w][kc];
                    qn = pos4[jn];
                    tn = type[jn];
                }
            }
            bool near = vj;
            if (vj && G.shift) {
                const float qx = q.x + ((code & 3) == 1 ? -L0 : ((code & 3) == 2 ? L0 : 0.0f));
                const float qy = q.y + (((code >> 2) & 3) == 1 ? -L1 : (((code >> 2) & 3) == 2 ? L1 : 0.0f));
                const float qz = q.z + (((code >> 4) & 3) == 1 ? -L2 : (((code >> 4) & 3) == 2 ? L2 : 0.0f));
                const float ex = fmaxf(fmaxf(bx0 - qx, qx - bx1), 0.0f);
                const float ey = fmaxf(fmaxf(by0 - qy, qy - by1), 0.0f);
                const float ez = fmaxf(fmaxf(bz0 - qz, qz - bz1), 0.0f);
                near = ex * ex + ey * ey + ez * ez < near_sq;
            }
            const unsigned nb = __ballot_sync(0xffffffffu, near);
            if (near) {
                const int pos = fill + __popc(nb & lt);
                s_fq[w][pos] = q;
                s_fe[w][pos] = (unsigned)j | ((unsigned)tj << MD_TYPE_SHIFT);
                s_fc[w][pos] = (unsigned char)code;
            }
            fill += __popc(nb);
            __syncwarp();
            if (fill >= 32) {
                process(32);
                /* move the overflow to the front of the queue */
                float4 tq;
                unsigned te = 0;
                unsigned char tc = 0;
                const bool mv = lane < fill - 32;
                if (mv) {
                    tq = s_fq[w][32 + lane];
                    te = s_fe[w][32 + lane];
                    tc = s_fc[w][32 + lane];
                }
                __syncwarp();
                if (mv) {
                    s_fq[w][lane] = tq;
                    s_fe[w][lane] = te;
                    s_fc[w][lane] = tc;
                }
                fill -= 32;
                __syncwarp();
            }
        }
        if (fill > 0) process(fill);
        /* pad every row to a multiple of 32 with the atom itself */
        for (int a = 0; a < ni; a++) {
            int c = __shfl_sync(0xffffffffu, mycnt, a);
            int lim = min(kp.cap, (c + MD_LIST_QUANTUM - 1) / MD_LIST_QUANTUM * MD_LIST_QUANTUM);
            int k = c + lane;
            if (k < lim) {
                int ta = type[i0 + a];
                nl[(size_t)(i0 + a) * kp.cap + k] = (unsigned)(i0 + a) | ((unsigned)ta << MD_TYPE_SHIFT);
            }
        }
        if (lane < ni) {
            int i = i0 + lane;
            nl_n[i] = mycnt < kp.cap ? mycnt : kp.cap;
            pos_old[i] = s_p[w][lane];
            if (mycnt > kp.cap) atomicMax(&st->list_overflow, mycnt);
        }
        __syncwarp();
    }
}

/* The warp-per-cell list builder.  A persistent grid (the blocks that fit
 * on the GPU at once): each warp takes the next cell from a counter in the
 * device state until none is left, so cells of uneven work balance, and a
 * launch without a rebuild due starts only that many blocks.  The counter
 * is reset by the pass that ends the rebuild. */
/* In a batch the warps take work items over the cells of the replicas that
 * rebuild only (a replica's cells are the contiguous ranks [cell0, cell0 +
 * ncells)): each block first scans, in shared memory, the cell counts of
 * those replicas, and maps a work item to its replica by binary search.  A
 * step in which a few replicas rebuild then costs one counter increment per
 * cell of those replicas, not one per cell of the batch (2.2 M atoms in
 * 230 k cells).  Batches of more than CW_MAXREP replicas take every cell and
 * skip the ones of replicas that keep their lists. */
constexpr int CW_MAXREP = 4 * CW_WARPS * 32;

__device__ __forceinline__ int rebuild_items(int nrep, const md_rep *__restrict__ reps,
                                             const int *__restrict__ rep_upd, int *s_pre)
{
    constexpr int K = CW_MAXREP / (CW_WARPS * 32);   /* replicas per thread */
    __shared__ int s_wsum[CW_WARPS];
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    int v[K], sum = 0;
#pragma unroll
    for (int k = 0; k < K; k++) {
        const int rr = t * K + k;
        v[k] = (rr < nrep && rep_upd[rr]) ? reps[rr].ncells : 0;
        sum += v[k];
    }
    int incl = sum;
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
    }
    if (lane == 31) s_wsum[w] = incl;
    __syncthreads();
    int before = incl - sum, total = 0;
    for (int u = 0; u < CW_WARPS; u++) {
        if (u < w) before += s_wsum[u];
        total += s_wsum[u];
    }
#pragma unroll
    for (int k = 0; k < K; k++) {
        const int rr = t * K + k;
        if (rr <= nrep) s_pre[rr] = before;   /* s_pre[nrep] = total */
        before += v[k];
    }
    __syncthreads();
    return total;
}

template <bool BATCH>
__global__ void __launch_bounds__(CW_WARPS * 32) k_build_cells(
    md_kparams kp, md_devstate *st, int always, int ncells, int nrep, const float4 *__restrict__ pos4,
    const int *__restrict__ type, const uint4 *__restrict__ excl_s,
    const int *__restrict__ cell_rank, const int *__restrict__ cell_lin,
    const int *__restrict__ cell_start, const unsigned *__restrict__ type_mask, unsigned *nl,
    int *nl_n, float4 *pos_old, const md_rep *__restrict__ reps, const int *__restrict__ crep,
    const int *__restrict__ rep_upd)
{
    pdl_wait();
    pdl_trigger();
    if (!always && !st->update) return;
    const int lane = threadIdx.x & 31;
    if (BATCH && nrep <= CW_MAXREP) {
        __shared__ int s_pre[CW_MAXREP + 1];
        const int items = rebuild_items(nrep, reps, rep_upd, s_pre);
        for (;;) {
            int wi = 0;
            if (lane == 0) wi = atomicAdd(&st->cell_next, 1);
            wi = __shfl_sync(0xffffffffu, wi, 0);
            if (wi >= items) break;
            int lo = 0, hi = nrep;   /* the replica: largest rr with s_pre[rr] <= wi */
            while (hi - lo > 1) {
                const int m = (lo + hi) >> 1;
                if (s_pre[m] <= wi) lo = m; else hi = m;
            }
            build_cell<BATCH>(reps[lo].cell0 + (wi - s_pre[lo]), kp, st, pos4, type, excl_s, cell_rank, cell_lin,
                              cell_start, type_mask, nl, nl_n, pos_old, reps, crep, rep_upd);
        }
        return;
    }
    for (;;) {
        int r = 0;
        if (lane == 0) r = atomicAdd(&st->cell_next, 1);
        r = __shfl_sync(0xffffffffu, r, 0);
        if (r >= ncells) break;
        build_cell<BATCH>(r, kp, st, pos4, type, excl_s, cell_rank, cell_lin, cell_start, type_mask, nl,
                          nl_n, pos_old, reps, crep, rep_upd);
    }
}

/* ---- The whole rebuild of a single system as one cooperative kernel ---- */

/* Grid-wide barrier of the cooperative rebuild (every block is resident:
 * the kernel is launched cooperatively).  The last block to arrive resets
 * the count and advances the generation; the others wait for the
 * generation to change for at most bar_ns of global time (MD_BAR_NS unless
 * a test shortens it), after which they record the timeout in st->status.
 * Returns false in every thread of the block when its wait timed out: the
 * caller then returns at once.  A block passes a barrier only when every
 * block has reached it, i.e. after every block finished the phase before
 * it, so no phase runs on counts or prefix sums a barrier did not complete;
 * blocks that passed while another one gave up find that one absent at the
 * next barrier and leave there.  The waiting
 * blocks poll the generation, which lies on another cache line than the
 * arrival counter, so the polls do not slow the arrivals' atomics (the two
 * on one line cost ~12 us per rebuild of 64000 ions with 1216 blocks of 4
 * warps, ~1 us with the 608 blocks of 8 warps used now; a two-level barrier
 * measured no faster). */
constexpr unsigned long long MD_BAR_NS = 50000000ull;   /* 50 ms */

__device__ __forceinline__ unsigned long long global_ns()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ bool grid_barrier(md_devstate *st, unsigned long long bar_ns)
{
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        volatile unsigned *gen = &st->bar_gen;
        const unsigned g = *gen;
        __threadfence();
        int ok = 1;
        if (atomicAdd(&st->bar_count, 1u) == gridDim.x - 1) {
            atomicExch(&st->bar_count, 0u);
            __threadfence();
            atomicAdd(&st->bar_gen, 1u);
        } else {
            const unsigned long long t0 = global_ns();
            while (*gen == g) {
                if (global_ns() - t0 > bar_ns) {
                    atomicOr(&st->status, 1);
                    ok = 0;
                    break;
                }
                __nanosleep(20);
            }
        }
        __threadfence();
        s_ok = ok;
    }
    __syncthreads();
    return s_ok != 0;
}

/* The order in which the list-building warps take the cells: most atoms
 * first (a counting sort of the cell ranks by atom count, counts above 63
 * together), so that the last cells handed out are the cheapest and the
 * warps finish close together.  Which warp builds a cell does not change
 * the cell's rows, so the order within a count may vary.  One block. */
__device__ __forceinline__ void work_order(int ncells, const int *cell_start, int *cell_work)
{
    __shared__ int s_at[64];
    if (threadIdx.x < 64) s_at[threadIdx.x] = 0;
    __syncthreads();
    for (int c = threadIdx.x; c < ncells; c += blockDim.x)
        atomicAdd(&s_at[min(cell_start[c + 1] - cell_start[c], 63)], 1);
    __syncthreads();
    if (threadIdx.x == 0) {
        int run = 0;
        for (int m = 63; m >= 0; m--) {
            const int h = s_at[m];
            s_at[m] = run;
            run += h;
        }
    }
    __syncthreads();
    for (int c = threadIdx.x; c < ncells; c += blockDim.x)
        cell_work[atomicAdd(&s_at[min(cell_start[c + 1] - cell_start[c], 63)], 1)] = c;
}

/* The arrays the rebuild passes touch. */
struct rb_ptrs {
    const int *cell_rank, *cell_lin;
    int *key, *cell_count, *cell_start, *cell_fill, *cell_work, *src;
    double *x, *v, *mass, *kick, *tmp_d;
    float4 *pos4, *tmp4, *pos_old;
    int *perm, *iperm, *type, *tmp_i;
    const uint4 *excl_orig;
    uint4 *excl_s;
    const int2 *bl_o;
    const int *bl_on;
    int2 *bl_s;
    int *bl_sn;
    const int4 *al_o;
    const int *al_on;
    int4 *al_s;
    int *al_sn;
    const unsigned *type_mask;
    unsigned *nl;
    int *nl_n;
    int ncells, has_bonds, has_angles;
    unsigned long long bar_ns;   /* limit of each barrier wait */
    int bar_drop;                /* test hook: this block leaves before the first barrier (-1: none) */
};

/* Binning, scan, scatter, in-cell order, permutation, remap, list build and
 * the closing reset in one launch, the passes separated by grid barriers;
 * a launch without a rebuild due returns at once.  128 threads per block,
 * the warp-per-cell builder (stencils of up to CW_MAXST cells). */
__global__ void __launch_bounds__(CW_WARPS * 32) k_rebuild_coop(md_kparams kp, md_devstate *st, int always,
                                                                rb_ptrs p)
{
    /* the same in every block: nothing writes either before the end; a
     * status left by an earlier launch (a barrier that timed out, whose
     * arrival count is then stale) stops every later rebuild */
    if (!always && !st->update) return;
    if (*(volatile int *)&st->status != 0) return;
    const int tid = blockIdx.x * blockDim.x + threadIdx.x, nth = gridDim.x * blockDim.x;
    const int n = kp.n;
    const unsigned long long bns = p.bar_ns;
    for (int i = tid; i < n; i += nth) key_one(kp, i, p.pos4, p.cell_rank, p.key, p.cell_count);
    if ((int)blockIdx.x == p.bar_drop) return;
    if (!grid_barrier(st, bns)) return;
    /* one block scans (one barrier is dearer than its few rounds) */
    if (blockIdx.x == 0) {
        const int total = scan_cells<CW_WARPS * 32>(p.ncells, p.cell_count, p.cell_start, p.cell_fill);
        if (threadIdx.x == 0) {
            p.cell_start[p.ncells] = total;
            st->builds += 1;
        }
        work_order(p.ncells, p.cell_start, p.cell_work);
    }
    if (!grid_barrier(st, bns)) return;
    for (int i = tid; i < n; i += nth) {
        const int r = p.key[i];
        p.src[p.cell_start[r] + atomicAdd(&p.cell_fill[r], 1)] = i;
    }
    if (!grid_barrier(st, bns)) return;
    {
        const int lane = threadIdx.x & 31, nw = nth >> 5;
        for (int c = tid >> 5; c < p.ncells; c += nw) {
            order_cell(c, p.cell_start, p.perm, p.src, nullptr, nullptr, lane);
            __syncwarp();
        }
    }
    if (!grid_barrier(st, bns)) return;
    for (int s = tid; s < n; s += nth)
        permute_one(kp, s, p.src, p.x, p.v, p.mass, p.kick, p.pos4, p.perm, p.type, p.tmp_d, p.tmp4, p.tmp_i);
    if (!grid_barrier(st, bns)) return;
    for (int s = tid; s < n; s += nth)
        copyback_one(kp, s, p.tmp_d, p.tmp4, p.tmp_i, p.x, p.v, p.mass, p.kick, p.pos4, p.perm, p.iperm, p.type);
    /* with bonds or angles the exclusions need the new order first; without,
     * the list build reads the sorted positions and types from the staging
     * arrays while the copy-back runs (it writes nothing the build reads) */
    const bool remap = p.has_bonds || p.has_angles;   /* the same in every block */
    if (remap) {
        if (!grid_barrier(st, bns)) return;
        for (int s = tid; s < n; s += nth)
            remap_one(kp, s, p.perm, p.iperm, p.excl_orig, p.excl_s, p.bl_o, p.bl_on, p.bl_s, p.bl_sn, p.al_o,
                      p.al_on, p.al_s, p.al_sn, p.has_bonds, p.has_angles);
        if (!grid_barrier(st, bns)) return;
    }
    {
        const float4 *bpos = remap ? p.pos4 : p.tmp4;
        const int *btype = remap ? p.type : p.tmp_i + kp.pitch;
        const int lane = threadIdx.x & 31;
        for (;;) {
            int r = 0;
            if (lane == 0) r = atomicAdd(&st->cell_next, 1);
            r = __shfl_sync(0xffffffffu, r, 0);
            if (r >= p.ncells) break;
            r = p.cell_work[r];
            build_cell<false>(r, kp, st, bpos, btype, p.excl_s, p.cell_rank, p.cell_lin, p.cell_start,
                              p.type_mask, p.nl, p.nl_n, p.pos_old, nullptr, nullptr, nullptr);
        }
    }
    if (!grid_barrier(st, bns)) return;
    if (tid == 0) {
        st->update = 0;
        st->cell_next = 0;
    }
}

}  // namespace

void launch_check(md_ctx *c, const md_kparams &kp)
{
    int nb = (kp.n + 255) / 256;
    if (c->batch) {
        k_check_b<<<nb, 256, 0, c->stream>>>(kp.n, c->reps_dev, c->arep, c->pos4, c->pos_old, c->st,
                                             c->rep_upd);
        return;
    }
    k_check<<<nb, 256, 0, c->stream>>>(kp, c->pos4, c->pos_old, c->st);
}

/* A pass of the rebuild: a plain launch, or (pdl) a programmatic dependent
 * launch whose blocks may be scheduled while the previous pass finishes;
 * every pass waits for its predecessor (pdl_wait) before it reads anything. */
template <typename... KArgs, typename... Args>
static void rb_launch(bool pdl, void (*k)(KArgs...), dim3 grid, dim3 block, cudaStream_t s,
                      Args... args)
{
    if (pdl) md_launch_pdl(k, grid, block, s, args...);
    else k<<<grid, block, 0, s>>>(args...);
}

/* Blocks of the persistent warp-per-cell builder: as many as are resident
 * at once (found once per context, on its first, uncaptured, build), at
 * most one warp per cell. */
static int cw_blocks(md_ctx *c, bool batch)
{
    int &g = c->cw_grid[batch ? 1 : 0];
    if (g == 0) {
        int dev = 0, nsm = 0, occ = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
        c->nsm = std::max(1, nsm);
        if (batch) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_build_cells<true>, CW_WARPS * 32, 0);
        else cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_build_cells<false>, CW_WARPS * 32, 0);
        g = std::max(1, nsm) * std::max(1, occ);
    }
    return std::max(1, std::min(g, (c->ncells + CW_WARPS - 1) / CW_WARPS));
}

/* Whether a single system rebuilds with the one-kernel rebuild: the
 * warp-per-cell builder with its stencil in shared memory, and enough
 * resident blocks found for a cooperative launch. */
bool md_rebuild_coop(md_ctx *c)
{
    if (c->batch || c->list_tpa != 0 || !c->rebuild_coop) return false;
    int nst = 1;
    for (int d = 0; d < 3; d++) nst *= c->stencil[d] < 0 ? c->ncell[d] : 2 * c->stencil[d] + 1;
    if (nst > CW_MAXST) return false;
    if (c->coop_grid == 0) {   /* found once, on the context's first, uncaptured, build */
        int dev = 0, nsm = 0, occ = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_rebuild_coop, CW_WARPS * 32, 0);
        c->coop_grid = occ > 0 ? nsm * occ : -1;
    }
    return c->coop_grid > 0;
}

void launch_rebuild(md_ctx *c, const md_kparams &kp, bool unconditional, bool all_replicas, bool pdl)
{
    int always = unconditional ? 1 : 0;
    if (c->batch) pdl = false;
    if (md_rebuild_coop(c)) {
        rb_ptrs p;
        p.cell_rank = c->cell_rank;
        p.cell_lin = c->cell_lin;
        p.key = c->key;
        p.cell_count = c->cell_count;
        p.cell_start = c->cell_start;
        p.cell_fill = c->cell_fill;
        p.cell_work = c->cell_work;
        p.src = c->src;
        p.x = c->x;
        p.v = c->v;
        p.mass = c->mass;
        p.kick = c->kick;
        p.tmp_d = c->tmp_d;
        p.pos4 = c->pos4;
        p.tmp4 = c->tmp4;
        p.pos_old = c->pos_old;
        p.perm = c->perm;
        p.iperm = c->iperm;
        p.type = c->type;
        p.tmp_i = c->tmp_i;
        p.excl_orig = c->excl_orig;
        p.excl_s = c->excl_s;
        p.bl_o = c->bl_o;
        p.bl_on = c->bl_on;
        p.bl_s = c->bl_s;
        p.bl_sn = c->bl_sn;
        p.al_o = c->al_o;
        p.al_on = c->al_on;
        p.al_s = c->al_s;
        p.al_sn = c->al_sn;
        p.type_mask = c->type_mask_dev;
        p.nl = c->nl;
        p.nl_n = c->nl_n;
        p.ncells = c->ncells;
        p.has_bonds = c->has_bonds;
        p.has_angles = c->has_angles;
        p.bar_ns = c->dbg_bar_ns > 0 ? c->dbg_bar_ns : MD_BAR_NS;
        p.bar_drop = c->dbg_bar_drop;
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(c->coop_grid);
        cfg.blockDim = dim3(CW_WARPS * 32);
        cfg.stream = c->stream;
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeCooperative;
        at[0].val.cooperative = 1;
        cfg.attrs = at;
        cfg.numAttrs = 1;
        const cudaError_t e = cudaLaunchKernelEx(&cfg, k_rebuild_coop, kp, c->st, always, p);
        if (e == cudaSuccess) return;
        /* a refused cooperative launch (fewer resident blocks than found
         * when the context was set up) falls back to the chain of passes,
         * for good when not capturing (during a capture the error stays
         * sticky in the capture, which then fails and is reported) */
        (void)cudaGetLastError();
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        cudaStreamIsCapturing(c->stream, &cs);
        if (cs != cudaStreamCaptureStatusNone) return;
        c->coop_grid = -1;
    }
    const int cwb = cw_blocks(c, c->batch);   /* also finds the SM count */
    int nb = (kp.n + 255) / 256;
    cudaStream_t s = c->stream;
    const bool batch = c->batch;
    const int rb = (c->nrep + 255) / 256;
    const int *arep = batch ? c->arep : nullptr;
    const int *crep = batch ? c->crep : nullptr;
    if (batch) {
        if (all_replicas) k_flag_all<<<rb, 256, 0, s>>>(c->rep_upd, c->nrep);
        k_cell_key_b<<<nb, 256, 0, s>>>(kp.n, kp.centered, c->reps_dev, c->arep, c->st, always, c->rep_upd,
                                        c->pos4, c->cell_rank, c->key, c->cell_count);
        k_cell_scan_b<<<(c->nrep + 7) / 8, 256, 0, s>>>(c->st, always, c->nrep, c->reps_dev,
                                                        c->rep_upd, c->cell_count, c->cell_start,
                                                        c->cell_fill);
    } else {
        rb_launch(pdl, k_cell_key, dim3(nb), dim3(256), s, kp, c->st, always, (const float4 *)c->pos4,
                  (const int *)c->cell_rank, c->key, c->cell_count);
        rb_launch(pdl, k_cell_scan, dim3(1), dim3(1024), s, kp, c->st, always, c->ncells, c->cell_count,
                  c->cell_start, c->cell_fill);
    }
    rb_launch(pdl, k_cell_scatter, dim3(nb), dim3(256), s, kp, (const md_devstate *)c->st, always,
              (const int *)c->key, (const int *)c->cell_start, c->cell_fill, c->src, arep,
              (const int *)c->rep_upd);
    /* a warp per cell, at most two blocks of 8 warps per SM (a loop over cells) */
    rb_launch(pdl, k_cell_order, dim3(std::min((c->ncells + 7) / 8, 2 * c->nsm)), dim3(256), s, kp,
              (const md_devstate *)c->st, always, c->ncells, (const int *)c->cell_start,
              (const int *)c->perm, c->src, crep, (const int *)c->rep_upd);
    rb_launch(pdl, k_permute, dim3(nb), dim3(256), s, kp, (const md_devstate *)c->st, always,
              (const int *)c->src, (const double *)c->x, (const double *)c->v,
              (const double *)c->mass, (const double *)c->kick, (const float4 *)c->pos4,
              (const int *)c->perm, (const int *)c->type, c->tmp_d, c->tmp4, c->tmp_i, arep,
              (const int *)c->rep_upd);
    rb_launch(pdl, k_copyback, dim3(nb), dim3(256), s, kp, (const md_devstate *)c->st, always,
              (const double *)c->tmp_d, (const float4 *)c->tmp4, (const int *)c->tmp_i, c->x, c->v,
              c->mass, c->kick, c->pos4, c->perm, c->iperm, c->type, arep, (const int *)c->rep_upd);
    /* exclusions and bonded lists to re-express only with bonds or angles
     * (in a batch every atom: a replica that kept its order maps to the
     * same lists) */
    if (c->has_bonds || c->has_angles)
        rb_launch(pdl, k_remap, dim3(nb), dim3(256), s, kp, (const md_devstate *)c->st, always,
                  (const int *)c->perm, (const int *)c->iperm, (const uint4 *)c->excl_orig, c->excl_s,
                  (const int2 *)c->bl_o, (const int *)c->bl_on, c->bl_s, c->bl_sn,
                  (const int4 *)c->al_o, (const int *)c->al_on, c->al_s, c->al_sn, c->has_bonds,
                  c->has_angles);
    if (batch) {
        /* at most 5 stencil cells per axis (cells of side >= rl/2): <= 125 */
        k_build_cells<true><<<cwb, CW_WARPS * 32, 0, s>>>(
            kp, c->st, always, c->ncells, c->nrep, c->pos4, c->type, c->excl_s, c->cell_rank, c->cell_lin,
            c->cell_start, c->type_mask_dev, c->nl, c->nl_n, c->pos_old, c->reps_dev, c->crep,
            c->rep_upd);
        k_clear_update_b<<<rb, 256, 0, s>>>(c->st, always, c->rep_upd, c->repst, c->nrep);
        return;
    }
    int ltpa = c->list_tpa;
    if (ltpa == 0) {   /* the warp-per-cell builder keeps up to 128 stencil cells in shared memory */
        int nst = 1;
        for (int d = 0; d < 3; d++) nst *= c->stencil[d] < 0 ? c->ncell[d] : 2 * c->stencil[d] + 1;
        if (nst > CW_MAXST) ltpa = 8;
    }
    long long threads = (long long)kp.n * (ltpa > 0 ? ltpa : 1);
    int lb = (int)((threads + 255) / 256);
    switch (ltpa) {
    case 0:
        rb_launch(pdl, k_build_cells<false>, dim3(cwb),
                  dim3(CW_WARPS * 32), s, kp, c->st, always, c->ncells, 0, (const float4 *)c->pos4,
                  (const int *)c->type, (const uint4 *)c->excl_s, (const int *)c->cell_rank,
                  (const int *)c->cell_lin, (const int *)c->cell_start,
                  (const unsigned *)c->type_mask_dev, c->nl, c->nl_n, c->pos_old,
                  (const md_rep *)nullptr, (const int *)nullptr, (const int *)nullptr);
        break;
#define MD_LIST_CASE(T)                                                                            \
    case T:                                                                                        \
        rb_launch(pdl, k_build_list<T>, dim3(lb), dim3(256), s, kp, c->st, always,                 \
                  (const float4 *)c->pos4, (const int *)c->type, (const uint4 *)c->excl_s,         \
                  (const int *)c->cell_rank, (const int *)c->cell_start,                           \
                  (const unsigned *)c->type_mask_dev, c->nl, c->nl_n, c->pos_old);                 \
        break;
        MD_LIST_CASE(1)
        MD_LIST_CASE(2)
        MD_LIST_CASE(4)
        MD_LIST_CASE(8)
        MD_LIST_CASE(16)
        MD_LIST_CASE(32)
#undef MD_LIST_CASE
    default:
        break;
    }
    rb_launch(pdl, k_clear_update, dim3(1), dim3(1), s, c->st);
}

void launch_set_condition(md_ctx *c, unsigned long long handle)
{
    k_set_condition<<<1, 1, 0, c->stream>>>((cudaGraphConditionalHandle)handle, c->st);
}
