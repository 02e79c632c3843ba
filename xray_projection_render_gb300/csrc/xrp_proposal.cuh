// xrp_proposal.cuh -- the proposal march: a learned proposal network plus
// distance certificates on top of the plain integrator.
//
// One warp marches one ray.  The ray's clipped sample range [k0, k1] (the
// same samples the plain integrator sums) is cut into segments of `mc`
// samples, 32 segments per round, one per lane.  Each lane evaluates the
// density and the certificate radius (margin32) at its segment's first
// sample; the segment's end point is the next segment's first sample.
// A segment is counted as (number of samples) x (density) when
//   (a) both end densities are certain and equal, and
//   (b) either the two certificate balls cover the segment (exact), or the
//       network's logit for the segment is at most tau (learned).
// Every other segment is integrated densely by the whole warp, sample by
// sample, exactly as the plain integrator does (FP32 guarded evaluation).
// The march writes optical depths; samples FP32 cannot decide go to a list
// that a second kernel evaluates in FP64 (reference arithmetic) and adds,
// and a third kernel forms exp(-T).  Keeping FP64 code out of the march
// keeps its register budget at two blocks per SM.
//
// Training data comes from the same march (TRAIN = true): every segment that
// (a) admits and (b)'s certificate does not settle is integrated densely and
// labelled 1 when any of its densities differs from the first (or is
// uncertain in FP32).
#pragma once
#include "xrp_train.cuh"

namespace xrp {

struct PropParams {
    const float* mlp;              // FP32 parameter block (MlpLayout); null: certificate only
    int mc;                        // samples per segment (multiple of 32)
    float tau;                     // logits above tau send a candidate to dense integration
    int refine;                    // 1: refine candidates by certificates; 0: dense
    int trace;                     // per-ray tracing (k_trace) instead: 1 ray/curve
                                   // certificates, 2 balls, 4 plain (every sample)
    int min_piece;                 // pieces of at most this many samples go dense
    float fc[3], fs[3];            // feature normalisation (p - fc) * fs
    const int* rays;               // optional ray list: (view, i, j) triples, views absolute
    int nrays;                     // number of listed rays
    unsigned long long* stats;     // optional counters, see kPropStat*
    // training rows (TRAIN): features, labels, capacity, row counter
    __nv_bfloat16* X;
    float* y;
    unsigned* count;
    unsigned cap;
    // samples left to FP64 (rendering): (ray, sample) pairs, counter,
    // capacity, and a flag raised when the list overflowed
    uint2* fb;
    unsigned* fb_count;
    unsigned fb_cap;
    unsigned* fb_overflow;
    // plain mode: rays to march again (a sample found the list full), one
    // slot per ray of a launch, and their counter
    unsigned* redo;
    unsigned* redo_count;
    unsigned redo_cap;
};

enum : int {
    kStatSegments = 0,  // segments visited
    kStatCertified,     // segments counted on their end-point certificate
    kStatRefined,       // pieces counted on a certificate during refinement
    kStatDense,         // pieces integrated densely
    kStatDenseSamples,  // samples evaluated by dense integration
    kStatEvaluations,   // certificate evaluations (density + radius)
    kStatFallbacks,     // samples re-evaluated in FP64
    kStatMlpRounds,     // warp-wide network evaluations (32 rows each)
    kStatRoutedDense,   // candidates the network sent to dense integration
    kStatSubdivided,    // candidates refined by certificates
    kStatOverflows,     // launches whose FP64 list overflowed (host; the call re-rendered plainly)
    kStatCount
};

// Per-warp work lists of the refinement: a stack of pieces (sample range
// [a, b] with the density and certificate radius at both ends, n samples
// counted) and a list of pieces to integrate densely.
constexpr int kStackCap = 128;
constexpr int kDenseCap = 160;
struct WarpLists {
    int a[kStackCap], b[kStackCap], n[kStackCap];
    float ra[kStackCap], ma[kStackCap], rb[kStackCap], mb[kStackCap];
    int da[kDenseCap], dn[kDenseCap];
};

constexpr int kPropWarps = 8;

struct PropShared {
    MlpShared W;
    __nv_bfloat16 rows[kPropWarps][32 * kMlpLd];
    WarpLists lists[kPropWarps];
    unsigned stats[kStatCount];
};

#if defined(__CUDACC__)

__device__ __forceinline__ void load_mlp_shared(const float* __restrict__ p, MlpShared& W) {
    for (int q = threadIdx.x; q < kMlpHid * kMlpIn; q += blockDim.x) {
        int o = q / kMlpIn, i = q % kMlpIn;
        W.w[0][o * kMlpLd + i] = __float2bfloat16_rn(p[MlpLayout::W1 + q]);
        W.w[1][o * kMlpLd + i] = __float2bfloat16_rn(p[MlpLayout::W2 + q]);
        W.w[2][o * kMlpLd + i] = __float2bfloat16_rn(p[MlpLayout::W3 + q]);
    }
    for (int q = threadIdx.x; q < kMlpHid; q += blockDim.x) {
        W.b[0][q] = p[MlpLayout::B1 + q];
        W.b[1][q] = p[MlpLayout::B2 + q];
        W.b[2][q] = p[MlpLayout::B3 + q];
        W.w4[q] = p[MlpLayout::W4 + q];
    }
    if (threadIdx.x == 0) W.b4 = p[MlpLayout::B4];
}

// Writes the feature row of segment (a, b) (world points) into `row`.
__device__ __forceinline__ void write_features(const PropParams& Q, const float* a, const float* b,
                                               __nv_bfloat16* row) {
    float an[3], bn[3];
#pragma unroll
    for (int c = 0; c < 3; c++) {
        an[c] = (a[c] - Q.fc[c]) * Q.fs[c];
        bn[c] = (b[c] - Q.fc[c]) * Q.fs[c];
    }
    segment_features(an, bn, [&](int k, float v) { row[k] = __float2bfloat16_rn(v); });
}

// Density and certificate radius at one point.  Not inlined: the march
// evaluates points at three places (segment ends, own end, refinement
// middles) and one shared body keeps the kernel inside the instruction
// cache; the hot dense loop keeps its own inlined density evaluation.
template <int DEPTH, bool DEFS>
__device__ __noinline__ float2 eval_dm(const SceneDev& S, float x, float y, float z) {
    float m;
    const float rho = dens_margin32<DEPTH, DEFS>(S, x, y, z, m);
    return make_float2(rho, m);
}

// Dense integration of the listed pieces, the warp's lanes over each
// piece's samples; undecided samples go to the FP64 list.
template <class Smp, class Count>
__device__ __forceinline__ void dense_pass(const WarpLists& ws, int nd, const Smp& smp, const Lattice& L,
                                           const PropParams& Q, long ray, KahanF& acc, Count& count) {
    const int lane = threadIdx.x & 31;
    count(kStatDense, (unsigned)nd);
    for (int q = 0; q < nd; q++) {
        const int a = ws.da[q], n = ws.dn[q];
        count(kStatDenseSamples, (unsigned)n);
        for (int k = a + lane; k < a + n; k += 32) {
            float rho = smp.f32(lattice_t(L, k));
            if (isunc(rho)) {
                unsigned slot = atomicAdd(Q.fb_count, 1u);
                if (slot < Q.fb_cap) Q.fb[slot] = make_uint2((unsigned)ray, (unsigned)k);
                rho = 0.0f;
            }
            acc.add(rho);
        }
    }
    __syncwarp();
}

// MODE: kPropDense (certificate, else dense), kPropRefine (certificate,
// else refinement), kPropNet (the network routes between the two),
// kPropTrain (training rows).  Each mode is its own kernel so none carries
// the others' code (instruction-cache pressure is this kernel's first stall).
enum : int { kPropDense = 0, kPropRefine = 1, kPropNet = 2, kPropTrain = 3 };

template <int DEPTH, bool DEFS, int MODE>
__global__ void __launch_bounds__(32 * kPropWarps, 2)
    k_propose(const __grid_constant__ SceneDev S, const __grid_constant__ Lattice L,
              const __grid_constant__ RenderParams P, const ViewDev* __restrict__ views, int view0,
              int nviews, const __grid_constant__ PropParams Q, float* __restrict__ out) {
    extern __shared__ __align__(16) unsigned char prop_smem[];
    PropShared& sh = *reinterpret_cast<PropShared*>(prop_smem);
    constexpr bool TRAIN = MODE == kPropTrain;
    constexpr bool REFINE = MODE == kPropRefine || MODE == kPropNet;
    constexpr bool use_mlp = MODE == kPropNet;
    if constexpr (use_mlp) load_mlp_shared(Q.mlp, sh.W);
    if (threadIdx.x < kStatCount) sh.stats[threadIdx.x] = 0;
    __syncthreads();
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    __nv_bfloat16* xrow = sh.rows[warp];
    WarpLists& ws = sh.lists[warp];
    const int res = P.res;
    const long img = (long)res * res;
    const long total = Q.rays ? (long)Q.nrays : (long)nviews * img;
    const long gw = (long)blockIdx.x * kPropWarps + warp;
    const long tw = (long)gridDim.x * kPropWarps;
    const bool stats = Q.stats != nullptr;
    // warp-aggregated counter update (lane 0 adds the warp's total)
    auto count = [&](int which, unsigned n) {
        if (stats && lane == 0 && n) atomicAdd(&sh.stats[which], n);
    };
    const int mc = Q.mc;

    // Rays go in batches of 32: each lane sets up one ray (the FP64 setup
    // runs once per ray, SIMT over the batch), then the warp marches the
    // batch's rays one after another, each cooperatively.
    for (long rb = gw * 32; rb < total; rb += tw * 32) {
        const long r = rb + lane;
        const bool rvalid = r < total;
        int v = 0, i = 0, j = 0;
        if (rvalid) {
            if (Q.rays) {
                v = Q.rays[3 * r];
                i = Q.rays[3 * r + 1];
                j = Q.rays[3 * r + 2];
            } else {
                v = view0 + (int)(r / img);
                long pix = r % img;
                i = (int)(pix / res);
                j = (int)(pix % res);
            }
        }
        Ray myray;
        int my_k0 = 0, my_k1 = -1;
        if (rvalid) {
            setup_ray_march(views[v], P, L, i, j, myray);
            float t0, t1;
            clip_ray(S.sup_lo, S.sup_hi, myray, t0, t1);
            if (!sample_range(L, t0, t1, L.K, my_k0, my_k1)) {
                my_k0 = 0;
                my_k1 = -1;
            }
        }
        float result = 0.0f;
        const int nb = (int)min((long)32, total - rb);
        for (int q = 0; q < nb; q++) {
            Ray ray;
#pragma unroll
            for (int c = 0; c < 3; c++) {
                ray.pc[c] = __shfl_sync(FULL, myray.pc[c], q);
                ray.d32[c] = __shfl_sync(FULL, myray.d32[c], q);
            }
            const int k0 = __shfl_sync(FULL, my_k0, q), k1 = __shfl_sync(FULL, my_k1, q);
            const int qv = __shfl_sync(FULL, v, q), qi = __shfl_sync(FULL, i, q),
                      qj = __shfl_sync(FULL, j, q);
            PixelRef px{views + qv, P.xs, qi, qj};
            SceneSampler<DEPTH, DEFS> smp{S, ray, px};
            KahanF acc;
            for (int base = k0; base <= k1; base += 32 * mc) {
                int a = base + lane * mc;
                const bool valid = a <= k1;
                if (!valid) a = k1;
                const int e = min(a + mc, k1 + 1);  // samples [a, e) belong to the segment
                const int ee = min(e, k1);          // end point of the certificate
                const float ta = lattice_t(L, a), te = lattice_t(L, ee);
                float pa[3], pe[3];
#pragma unroll
                for (int c = 0; c < 3; c++) {
                    pa[c] = fmaf(ray.d32[c], ta, ray.pc[c]);
                    pe[c] = fmaf(ray.d32[c], te, ray.pc[c]);
                }
                float rho_a = 0.0f, m_a = 0.0f;
                if (valid) {
                    const float2 dm = eval_dm<DEPTH, DEFS>(S, pa[0], pa[1], pa[2]);
                    rho_a = dm.x;
                    m_a = dm.y;
                }
                float rho_e = __shfl_down_sync(FULL, rho_a, 1);
                float m_e = __shfl_down_sync(FULL, m_a, 1);
                const bool own_end = valid && (lane == 31 || a + mc > k1);
                if (own_end) {
                    const float2 dm = eval_dm<DEPTH, DEFS>(S, pe[0], pe[1], pe[2]);
                    rho_e = dm.x;
                    m_e = dm.y;
                }
                const unsigned nvalid = __popc(__ballot_sync(FULL, valid));
                count(kStatSegments, nvalid);
                count(kStatEvaluations, nvalid + __popc(__ballot_sync(FULL, own_end)));
                const bool same = valid && !isunc(rho_a) && !isunc(rho_e) && rho_a == rho_e;
                const bool cert = same && (m_a + m_e >= (float)(ee - a) * L.ds32 * 1.00001f);
                const bool cand = same && !cert;  // refined by certificates or densely
                if constexpr (TRAIN) {
                    // label each candidate: does any of its densities differ?
                    if (cand) write_features(Q, pa, pe, xrow + lane * kMlpLd);
                    __syncwarp();
                    unsigned mask = __ballot_sync(FULL, cand);
                    while (mask) {
                        const int s = __ffs(mask) - 1;
                        mask &= mask - 1;
                        const int sa = __shfl_sync(FULL, a, s), se = __shfl_sync(FULL, e, s);
                        const float rho0 = __shfl_sync(FULL, rho_a, s);
                        bool differs = false;
                        for (int k = sa + 1 + lane; k < se; k += 32) {
                            float rho = smp.f32(lattice_t(L, k));
                            differs |= isunc(rho) || rho != rho0;
                        }
                        const bool lab = __any_sync(FULL, differs);
                        unsigned slot = 0;
                        if (lane == s) slot = atomicAdd(Q.count, 1u);
                        slot = __shfl_sync(FULL, slot, s);
                        if (slot < Q.cap) {
                            const uint32_t* src = reinterpret_cast<const uint32_t*>(xrow + s * kMlpLd);
                            uint32_t* dst = reinterpret_cast<uint32_t*>(Q.X + (size_t)slot * kMlpIn);
                            dst[lane] = src[lane];
                            if (lane == 0) Q.y[slot] = lab ? 1.0f : 0.0f;
                        }
                    }
                    __syncwarp();
                } else {
                    // the network routes candidates: likely transitions -> dense,
                    // the rest -> refinement by certificates
                    bool to_dense = cand && !REFINE;
                    if constexpr (use_mlp) {
                        if (__any_sync(FULL, cand)) {
                            write_features(Q, pa, pe, xrow + lane * kMlpLd);
                            __syncwarp();
                            float logit = mlp_forward_warp(sh.W, xrow);
                            __syncwarp();
                            to_dense = cand && logit > Q.tau;
                            count(kStatMlpRounds, 1);
                        }
                    }
                    if (cert) acc.add(rho_a * (float)(e - a));
                    count(kStatCertified, __popc(__ballot_sync(FULL, cert)));
                    const bool sub = cand && !to_dense;
                    const bool dense = valid && !cert && !sub;
                    const unsigned smask = __ballot_sync(FULL, sub), dmask = __ballot_sync(FULL, dense);
                    count(kStatRoutedDense, __popc(__ballot_sync(FULL, cand && to_dense && use_mlp)));
                    count(kStatSubdivided, __popc(smask));
                    const unsigned lt = (1u << lane) - 1u;
                    // the stack and the dense list are empty at this point
                    if (sub) {
                        const int q2 = __popc(smask & lt);
                        ws.a[q2] = a;
                        ws.b[q2] = ee;
                        ws.n[q2] = e - a;
                        ws.ra[q2] = rho_a;
                        ws.ma[q2] = m_a;
                        ws.rb[q2] = rho_e;
                        ws.mb[q2] = m_e;
                    }
                    if (dense) {
                        const int q2 = __popc(dmask & lt);
                        ws.da[q2] = a;
                        ws.dn[q2] = e - a;
                    }
                    int sp = REFINE ? __popc(smask) : 0, nd = __popc(dmask);
                    __syncwarp();
                    // refinement waves: split each piece at its middle sample,
                    // certify the halves, push the rest (dense below min_piece)
                    while (REFINE && sp > 0) {
                        if (nd > kDenseCap - 64) {
                            dense_pass(ws, nd, smp, L, Q, rb + q, acc, count);
                            nd = 0;
                        }
                        const int take = min(sp, 32);
                        sp -= take;
                        const bool have = lane < take;
                        int pa_ = 0, pb_ = 0, pn = 0;
                        float pra = 0.f, pma = 0.f, prb = 0.f, pmb = 0.f;
                        if (have) {
                            pa_ = ws.a[sp + lane];
                            pb_ = ws.b[sp + lane];
                            pn = ws.n[sp + lane];
                            pra = ws.ra[sp + lane];
                            pma = ws.ma[sp + lane];
                            prb = ws.rb[sp + lane];
                            pmb = ws.mb[sp + lane];
                        }
                        __syncwarp();
                        const int mid = (pa_ + pb_) >> 1;
                        float rm = 0.0f, mm = 0.0f;
                        if (have) {
                            const float tm = lattice_t(L, mid);
                            const float x = fmaf(ray.d32[0], tm, ray.pc[0]);
                            const float y = fmaf(ray.d32[1], tm, ray.pc[1]);
                            const float z = fmaf(ray.d32[2], tm, ray.pc[2]);
                            const float2 dm = eval_dm<DEPTH, DEFS>(S, x, y, z);
                            rm = dm.x;
                            mm = dm.y;
                        }
                        count(kStatEvaluations, (unsigned)take);
                        const int nl = mid - pa_, nr = pn - nl;
                        const bool mok = have && !isunc(rm);
                        const bool lcert = mok && rm == pra && pma + mm >= (float)(mid - pa_) * L.ds32 * 1.00001f;
                        const bool rcert = mok && rm == prb && mm + pmb >= (float)(pb_ - mid) * L.ds32 * 1.00001f;
                        if (lcert) acc.add(pra * (float)nl);
                        if (rcert) acc.add(prb * (float)nr);
                        count(kStatRefined, __popc(__ballot_sync(FULL, lcert)) + __popc(__ballot_sync(FULL, rcert)));
                        // children: split further while long enough, else dense
                        const bool room = sp + 2 * take <= kStackCap;
                        const bool lsplit = have && !lcert && mok && nl > Q.min_piece && room;
                        const bool rsplit = have && !rcert && mok && nr > Q.min_piece && room;
                        const bool ldense = have && !lcert && !lsplit && nl > 0;
                        const bool rdense = have && !rcert && !rsplit && nr > 0;
                        const unsigned mls = __ballot_sync(FULL, lsplit), mrs = __ballot_sync(FULL, rsplit);
                        const unsigned mld = __ballot_sync(FULL, ldense), mrd = __ballot_sync(FULL, rdense);
                        if (lsplit) {
                            const int q2 = sp + __popc(mls & lt);
                            ws.a[q2] = pa_; ws.b[q2] = mid; ws.n[q2] = nl;
                            ws.ra[q2] = pra; ws.ma[q2] = pma; ws.rb[q2] = rm; ws.mb[q2] = mm;
                        }
                        if (rsplit) {
                            const int q2 = sp + __popc(mls) + __popc(mrs & lt);
                            ws.a[q2] = mid; ws.b[q2] = pb_; ws.n[q2] = nr;
                            ws.ra[q2] = rm; ws.ma[q2] = mm; ws.rb[q2] = prb; ws.mb[q2] = pmb;
                        }
                        if (ldense) {
                            const int q2 = nd + __popc(mld & lt);
                            ws.da[q2] = pa_;
                            ws.dn[q2] = nl;
                        }
                        if (rdense) {
                            const int q2 = nd + __popc(mld) + __popc(mrd & lt);
                            ws.da[q2] = mid;
                            ws.dn[q2] = nr;
                        }
                        sp += __popc(mls) + __popc(mrs);
                        nd += __popc(mld) + __popc(mrd);
                        __syncwarp();
                    }
                    if (nd) dense_pass(ws, nd, smp, L, Q, rb + q, acc, count);
                }
            }
            if constexpr (!TRAIN) {
                float sum = acc.s - acc.c;
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(FULL, sum, o);
                if (lane == q) {
                    float w = P.density_multiplier * L.ds32;
                    result = fmaf(w, sum, P.flat_field);  // optical depth; exp in k_prop_finish
                }
            }
        }
        if constexpr (!TRAIN) {
            if (rvalid) out[r] = result;
        }
    }
    if (stats) {
        __syncthreads();
        if (threadIdx.x < kStatCount && sh.stats[threadIdx.x])
            atomicAdd(&Q.stats[threadIdx.x], (unsigned long long)sh.stats[threadIdx.x]);
    }
}

// Certificate tracing: one thread per ray (16x16 pixel tiles, warps of 8x4
// pixels like k_render, so neighbouring rays stay coherent).  At sample k
// the density and the certificate radius m are evaluated; samples k .. k+j
// with j*ds <= m lie inside the ball around sample k, so they all have its
// density and are counted at once, and the march jumps to k+j+1.  Far from
// any boundary the jumps are long; approaching one they shrink
// geometrically; next to it the march steps sample by sample.  RAY (affine
// deformation chains): the certificate is the ray bound of dens_ray32, the
// distance along the ray to the next possible density change, so a ray
// jumps straight to the next boundary instead of approaching it.  CURVE
// (smooth non-affine chains): the certificate is the curve bound of
// dens_curve32, the first parameter at which the curved path of the
// deformed samples can reach a boundary.  CERT: 0 ball, 1 ray, 2 curve,
// 3 curve for scenes whose leaves are all gyroids (a smaller kernel), 4 no
// certificate: the plain integrator, every sample evaluated.
// Samples FP32 cannot decide go to the FP64 list like the other march modes
// (in the plain mode a ray with a sample that found the list full is marched
// again by k_plain_redo, so the plain integrator never needs the host's
// overflow check).
// Resident blocks per SM for depth < 3, measured: 4 (64 registers; lattice
// with ray bounds 415 against 382 Mrays/s with 3 and 410 with 5, gyroid with
// balls 1462 against 1406 with 3).  Tried and dropped: four pixels per
// thread in one flattened loop (a lane starts its next ray when one ends, to
// recover the ~13 % of lane slots lost to warps' longest rays): the lanes'
// rays drift apart and evaluations diverge, lattice 464 -> 411 Mrays/s,
// gyroid 2041 -> 1396.
// Resident blocks per SM of the tracing kernel with curve certificates
// (depth < 3): its Jacobian-vector products and quadratic bounds need more
// registers than the ball and ray variants (at 64 registers ptxas spills
// about 370 bytes per thread on the gyroid's depth-1 kernel, at 80 about 240).
#ifndef XRP_CURVE_MIN_BLOCKS
#define XRP_CURVE_MIN_BLOCKS 4
#endif
// Pixel columns of a warp's tile in the tracing kernel (8: 8 x 4 pixels;
// 4 x 8 and 16 x 2 measured the same within 1 %: lattice 534 / 528 against
// 534, gyroid 2042 / 2048 against 2035 Mrays/s).
#ifndef XRP_TRACE_TILE_W
#define XRP_TRACE_TILE_W 8
#endif
// The plain mode reads the node table from shared memory (1) or through L1
// (0: lattice 164.6 against 167.8 Mrays/s, gyroid 109.3 against 111.8).
#ifndef XRP_PLAIN_SMEM_NODES
#define XRP_PLAIN_SMEM_NODES 1
#endif
// Resident blocks per SM of the plain mode (depth < 3; three blocks ran
// 151 against 159 Mrays/s on the lattice, five 161 against 168, gyroid
// 106 against 112).
#ifndef XRP_PLAIN_MIN_BLOCKS
#define XRP_PLAIN_MIN_BLOCKS 4
#endif
// Resident blocks per SM of the hierarchical integrator (depth < 3; three
// blocks measured slower: lattice 87 / plain 60 / gyroid 394 against
// 92 / 66 / 418 Mrays/s).
#ifndef XRP_HIER_MIN_BLOCKS
#define XRP_HIER_MIN_BLOCKS 4
#endif
template <int DEPTH, bool DEFS, bool HIER, int CERT>
__global__ void __launch_bounds__(256, DEPTH >= 3 ? 2
                                       : HIER     ? XRP_HIER_MIN_BLOCKS
                                       : (CERT == 2 || CERT == 3) ? XRP_CURVE_MIN_BLOCKS
                                       : CERT == 4                ? XRP_PLAIN_MIN_BLOCKS
                                                                  : 4)
    k_trace(const __grid_constant__ SceneDev S, const __grid_constant__ Lattice L,
            const __grid_constant__ RenderParams P, const ViewDev* __restrict__ views, int view0, int nviews,
            const __grid_constant__ PropParams Q, float* __restrict__ out) {
    constexpr bool RAY = CERT == 1, CURVE = CERT == 2 || CERT == 3, PLAIN = CERT == 4;
    constexpr int LM = CERT == 3 ? kLeafGyroid : kLeafAll;
    const int res = P.res;
    const int tpr = (res + 15) >> 4;
    const int tpv = tpr * tpr;
    const int b = blockIdx.x;
    const int v = b / tpv;
    const int t = b - v * tpv;
    const int ti = t / tpr, tj = t - ti * tpr;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    // a warp renders XRP_TRACE_TILE_W x (32 / XRP_TRACE_TILE_W) pixels of the
    // block's 16 x 16
    constexpr int TW = XRP_TRACE_TILE_W, TH = 32 / TW, WX = 16 / TW;
    const int i = (ti << 4) + (warp / WX) * TH + lane / TW;
    const int j = (tj << 4) + (warp % WX) * TW + lane % TW;
    unsigned evals = 0, inplace = 0;  // evaluations; FP64 re-evaluations in place
    bool lost = false;                // a sample found the FP64 list full
    // the scene's node table in shared memory (S.nnodes > 0: it fits); the
    // FP64 re-evaluation keeps the global table
    extern __shared__ __align__(16) unsigned char trace_smem[];
    SceneDev Sl = S;
    if (S.nnodes > 0 && (!PLAIN || XRP_PLAIN_SMEM_NODES)) {
        const int4* src = reinterpret_cast<const int4*>(S.nodes);
        int4* dst = reinterpret_cast<int4*>(trace_smem);
        for (int q = threadIdx.x; q < S.nnodes * (int)(sizeof(Node) / sizeof(int4)); q += blockDim.x)
            dst[q] = src[q];
        __syncthreads();
        Sl.nodes = reinterpret_cast<const Node*>(trace_smem);
    }
    const bool valid = v < nviews && i < res && j < res;
    const long r = ((long)v * res + i) * res + j;
    const ViewDev& V = views[view0 + (valid ? v : 0)];
    Ray ray;
    int k0 = 0, k1 = -1;
    bool has = false;  // the ray meets the support
    if (valid) {
        setup_ray_march(V, P, L, i, j, ray);
        float t0, t1;
        clip_ray(S.sup_lo, S.sup_hi, ray, t0, t1);
        has = sample_range(L, t0, t1, L.K, k0, k1);
    }
    float sum = 0.0f;
    if constexpr (HIER) {
        // a coarse sample's value decides refinement: FP64 in place, with
        // certificates the warp's waiting lanes served together (wm: the
        // lanes marching; 4 lanes / 32 iterations measured best: lattice
        // 76 -> 92 Mrays/s, gyroid 369 -> 413; the plain march, whose lanes
        // stay in step, gained nothing: 64.4 -> 62.9); fine samples only
        // add, so they go to the list (high bit)
        const unsigned wm = __ballot_sync(0xffffffffu, has);
        if (has)
            sum = trace_sum_hier<DEPTH, DEFS, RAY, CURVE, LM, PLAIN, !PLAIN>(
                Sl, L, ray, k0, k1,
                [&](int q, bool fine) {
                    if (!fine) {
                        inplace++;
                        return (float)sample64_pixel(S, V, P.xs, i, j, L.s64[q]);
                    }
                    unsigned slot = atomicAdd(Q.fb_count, 1u);
                    if (slot < Q.fb_cap) Q.fb[slot] = make_uint2((unsigned)r, (unsigned)q | 0x80000000u);
                    else lost = true;
                    return 0.0f;
                },
                evals, wm);
    } else if (has) {
        auto unc = [&](int k) {
            unsigned slot = atomicAdd(Q.fb_count, 1u);
            if (slot < Q.fb_cap) Q.fb[slot] = make_uint2((unsigned)r, (unsigned)k);
            else lost = true;
            return 0.0f;
        };
        if constexpr (PLAIN) sum = plain_sum<DEPTH, DEFS>(Sl, L, ray, k0, k1, unc, evals);
        else sum = trace_sum<DEPTH, DEFS, RAY, CURVE, LM>(Sl, L, ray, k0, k1, unc, evals);
    }
    if (valid) {
        const float w = HIER ? P.density_multiplier : P.density_multiplier * L.ds32;
        out[r] = fmaf(w, sum, P.flat_field);
        if constexpr (PLAIN) {
            // a sample found the list full: the whole ray is marched again
            // (k_plain_redo, after the FP64 pass); the redo list holds every
            // ray of the launch
            if (lost) {
                const unsigned q = atomicAdd(Q.redo_count, 1u);
                if (q < Q.redo_cap) Q.redo[q] = (unsigned)r;
            }
        }
    }
    if (Q.stats) {
        unsigned s = __reduce_add_sync(0xffffffffu, evals);
        if (lane == 0 && s) atomicAdd(&Q.stats[kStatEvaluations], (unsigned long long)s);
        if constexpr (HIER) {
            unsigned f = __reduce_add_sync(0xffffffffu, inplace);
            if (lane == 0 && f) atomicAdd(&Q.stats[kStatFallbacks], (unsigned long long)f);
        }
    }
}

#if defined(XRP_PROP_RENDER_KERNELS)
// FP64 re-evaluation of the samples the march left undecided: adds
// w * density (reference arithmetic at the reference's position) to the
// ray's optical depth.  Rays are numbered within the launch (view0 first).
// Four blocks per SM (64 registers): a block fits the registers one block of
// the tracing kernel frees, so the FP64 pass of one launch group can run
// beside the next group's march.
#ifndef XRP_FB_MIN_BLOCKS
#define XRP_FB_MIN_BLOCKS 4
#endif
__global__ void __launch_bounds__(256, XRP_FB_MIN_BLOCKS)
    k_prop_fallback(const __grid_constant__ SceneDev S, const __grid_constant__ Lattice L,
                    const __grid_constant__ RenderParams P, const ViewDev* __restrict__ views,
                    int view0, const uint2* __restrict__ fb, const unsigned* __restrict__ fb_count,
                    unsigned fb_cap, float* __restrict__ T, unsigned long long* __restrict__ stats,
                    unsigned* __restrict__ overflow) {
    const unsigned total = *fb_count;
    const unsigned n = min(total, fb_cap);
    if (blockIdx.x == 0 && threadIdx.x == 0 && total > fb_cap) atomicOr(overflow, 1u);
    const long img = (long)P.res * P.res;
    const float w = P.density_multiplier * L.ds32;
    const float wf = P.density_multiplier * L.dsf32;  // fine samples (hierarchical)
    for (unsigned q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
        const uint2 e = fb[q];
        const long r = e.x;
        const int v = view0 + (int)(r / img);
        const long pix = r % img;
        const int i = (int)(pix / P.res), j = (int)(pix % P.res);
        const bool fine = (e.y & 0x80000000u) != 0;
        const unsigned idx = e.y & 0x7fffffffu;
        double rho = sample64_pixel_inl(S, views[v], P.xs, i, j, fine ? L.f64[idx] : L.s64[idx]);
        atomicAdd(&T[r], (fine ? wf : w) * (float)rho);
    }
    if (stats && blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(&stats[kStatFallbacks], (unsigned long long)n);
}

// Transmittance exp(-T) of every ray of a launch.
__global__ void k_prop_finish(float* __restrict__ T, long n) {
    for (long q = (long)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x)
        T[q] = expf(-T[q]);
}
#endif  // XRP_PROP_RENDER_KERNELS



#endif  // __CUDACC__

}  // namespace xrp
