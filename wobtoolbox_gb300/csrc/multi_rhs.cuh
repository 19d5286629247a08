// Multi-RHS walks: up to 64 boundary-data right-hand sides (RHS) share one set of paths.
//
// The backward estimators whose sampling ignores the boundary data -- single layer with uniform or
// RIS sampling (estimator.cuh:276-334) and direct with two uniform samples per bounce
// (estimator.cuh:335-347) -- give a path value that is linear in the data. Every data-dependent
// operation of the scalar walk (contrib = contrib + w * fbk(...) in the bounce loop, out = sdk(...) +
// mu * sdu(...) at the evaluation point) is a fixed function of the data at one or two visited
// boundary points, with scalar weights that do not depend on the data.
//
// Each lane walks one path with the scalar walker's code. At every bounce it writes one tape entry
// (the weights it computed and references -- element and interpolation weights -- to the points
// whose data the bounce reads) to a per-warp slot in shared memory; the warp then replays the
// bounce's 32 entries for every RHS, lane l owning RHS l and l + 32, so the data rows of one
// element (R consecutive floats per vertex) are read with coalesced loads. The replay performs the
// scalar walk's float operations in the same order, so the value of a path for RHS r is
// bit-identical to the scalar walk on the data of RHS r; only the data reads are per RHS.
//
// The per-path accumulators live in shared memory ([32 paths][64 RHS] floats per warp). Sums are
// FP64 per (point, RHS), added once per warp unit.
//
// With a control variate cv (piecewise constant per stored element, one column per RHS; no
// counterpart in the reference) the domain estimate becomes
//   u(x) = sdk(x, y1) + (mu(y0) - cv(y0)) sdu(x, y0) + sum_{i < n} (sdu(x, z_i) / n) cv(z_i),
// unbiased for any cv: the z_i are n uniform boundary samples drawn after the walk, so the walk
// itself (and mu) is the plain estimator's. The potential samples go through the same tape.
#pragma once

#include "kernels.cuh"
#include "multi_rhs.hpp"

namespace wobgb {
namespace mrhs {

constexpr uint32_t kRefInput = 0xFFFFFFFFu;  // the evaluation point's own data (boundary input)
constexpr uint32_t kRefZero = 0xFFFFFFFEu;   // the zero point an empty RIS selection returns

// A visited boundary point: stored element and the interpolation weights of its data
// (2D: k0 = u along the segment; 3D: the three barycentric weights of uniform_point).
struct PRef {
    uint32_t e;
    float k0, k1, k2;
};

enum : int { kFormA = 0, kFormB = 1, kFormC = 2, kFormD = 3 };

// One bounce of one path: T(data) = form(c, k, data(a), data(b)); contrib = contrib + w * T.
//   A: c * (a + 0)             single layer fbk (bie_models.cuh:245-257)
//   B: c * ((a + 0) + k * (b + 0))   direct fbk, x and y Dirichlet (bie_models.cuh:480-492)
//   C: c * ((a + 0) - k * (b + 0))   direct fbk, x Dirichlet, y Neumann / Robin
//   D: k * (b + 0)             direct fbk, x Neumann / Robin
// The "+ 0" terms are the absent source term of the scalar walk, kept so the operations match.
struct __align__(16) TapeEntry {
    float w, c, k;
    int form;
    PRef a, b;
};

template <int D> __device__ __forceinline__ PRef uniform_ref(uint32_t idx, const float *u) {
    PRef r;
    r.e = idx;
    if constexpr (D == 2) {
        r.k0 = u[1];
        r.k1 = 0.0f;
        r.k2 = 0.0f;
    } else {
        const float sq = sqrtf(u[1]);
        r.k0 = 1.0f - sq;
        r.k1 = sq * (1.0f - u[2]);
        r.k2 = u[2] * sq;
    }
    return r;
}

// sample_uniform / sample_uniform_pair that also return the references of their points.
template <int D> __device__ __forceinline__ BPoint<D> sample_uniform_ref(const SceneView<D> &s, PathRng &rng, float &inv_pdf,
                                                                        PRef &ref) {
    float u[D];
#pragma unroll
    for (int i = 0; i < D; i++) u[i] = rng.uniform();
    const uint32_t idx = cdf_search(s.area_cdf, s.area_guide, s.area_G, u[0]);
    inv_pdf = s.total_area;
    ref = uniform_ref<D>(idx, u);
    return uniform_point<D>(load_elem<D>(s, idx), u);
}
template <int D> __device__ __forceinline__ void sample_uniform_pair_ref(const SceneView<D> &s, PathRng &rng, BPoint<D> &ya,
                                                                        float &ipa, PRef &ra, BPoint<D> &yb, float &ipb,
                                                                        PRef &rb) {
    float ua[D], ub[D];
#pragma unroll
    for (int i = 0; i < D; i++) ua[i] = rng.uniform();
#pragma unroll
    for (int i = 0; i < D; i++) ub[i] = rng.uniform();
    const uint4 ga = __ldg(s.area_guide + guide_bin(s.area_G, ua[0]));
    const uint4 gb = __ldg(s.area_guide + guide_bin(s.area_G, ub[0]));
    const uint32_t ia = cdf_resolve(s.area_cdf, ga, ua[0]);
    const uint32_t ib = cdf_resolve(s.area_cdf, gb, ub[0]);
    const Elem<D> ea = load_elem<D>(s, ia);
    const Elem<D> eb = load_elem<D>(s, ib);
    ya = uniform_point<D>(ea, ua);
    yb = uniform_point<D>(eb, ub);
    ra = uniform_ref<D>(ia, ua);
    rb = uniform_ref<D>(ib, ub);
    ipa = s.total_area;
    ipb = s.total_area;
}

template <int D, int kBie, int kStrat> struct MultiWalker : Walker<D, kBie, kStrat, false> {
    using Base = Walker<D, kBie, kStrat, false>;
    __device__ __forceinline__ MultiWalker(const SceneView<D> &s_, const WalkParams &p_, uint32_t stream, uint32_t point,
                                           uint64_t path)
        : Base(s_, p_, stream, point, path) {}

    // Walker::sample_ris with the reference of the selected candidate.
    __device__ __forceinline__ BPoint<D> sample_ris_ref(const BPoint<D> &yp, float &inv_pdf, PRef &ref) {
        uint32_t sel, M;
        float su[D], w_sum;
        this->ris_select(yp, sel, su, w_sum, M);
        BPoint<D> y;
        if (sel != 0xFFFFFFFFu) {
            y = uniform_point<D>(load_elem<D>(this->s, sel), su);
            ref = uniform_ref<D>(sel, su);
        } else {
            y = bp_zero<D>();
            ref.e = kRefZero;
            ref.k0 = ref.k1 = ref.k2 = 0.0f;
        }
        inv_pdf = w_sum / fmax_ref(this->ris_target(yp.type, yp, y) * (float)M, kEps10);
        return y;
    }

    // One iteration of unknown_boundary's loop for the point yprev (reference yref) with weight wgt
    // (already halved on the last bounce): fills the tape entry, advances yprev / yref / wgt.
    // last: the path's final bounce, whose transport (next sample and weight) is never used and
    // is skipped, as in the scalar walk.
    __device__ __forceinline__ void bounce(BPoint<D> &yprev, PRef &yref, float &wgt, TapeEntry &e, bool last) {
        e.w = wgt;
        e.a = yref;
        if constexpr (kStrat == kStratSingleLayer) {
            e.form = kFormA;
            e.k = 0.0f;
            e.b = yref;
            e.c = (yprev.type == kDirichlet) ? 2.0f * this->p.fk : this->dtc() / this->ift(yprev.angle);
            if (last) return;
            BPoint<D> y;
            float ip;
            PRef r;
            if (this->p.n_resampling == 1) y = sample_uniform_ref<D>(this->s, this->rng, ip, r);
            else y = sample_ris_ref(yprev, ip, r);
            wgt = wgt * this->fbu(yprev, y, ip, true);
            if (this->stayed) r = yref;
            yprev = y;
            yref = r;
        } else {
            BPoint<D> ya, y;
            float ipa, ip;
            PRef ra, r;
            if (last) ya = sample_uniform_ref<D>(this->s, this->rng, ipa, ra);
            else sample_uniform_pair_ref<D>(this->s, this->rng, ya, ipa, ra, y, ip, r);
            const BPoint<D> &x = yprev;
            e.b = ra;
            if (x.type == kDirichlet) {
                e.c = this->dtc() * this->p.fk;
                if (ya.type == kDirichlet) {
                    e.k = this->dtc() / this->ift(x.angle) * ipa * this->K.dG_dny(ya.p, x.p, ya.n);
                    e.form = kFormB;
                } else {
                    e.k = this->dtc() / this->ift(x.angle) * ipa * this->K.G(ya.p, x.p);
                    e.form = kFormC;
                }
            } else {
                e.c = 0.0f;
                if (ya.type == kDirichlet) e.k = -this->dtc() / this->ift(x.angle) * ipa * this->K.dG_dny(ya.p, x.p, ya.n);
                else e.k = this->dtc() / this->ift(x.angle) * ipa * this->K.G(ya.p, x.p);
                e.form = kFormD;
            }
            if (last) return;
            wgt = wgt * this->fbu(yprev, y, ip, true);
            if (this->stayed) r = yref;
            yprev = y;
            yref = r;
        }
    }
};

template <int D> struct RhsData {
    const float *__restrict__ table;  // [n_elems][D][R], storage order
    const float *__restrict__ input;  // [n_points][R]: data of the boundary evaluation points
    const float *__restrict__ cv;     // [n_elems][R]: control variate per stored element (or null)
    uint32_t R, n_pot;

    __device__ __forceinline__ float at(const PRef &r, uint32_t pt, uint32_t c) const {
        if (r.e == kRefInput) return __ldg(input + (size_t)pt * R + c);
        if (r.e == kRefZero) return 0.0f;
        const float *q = table + (size_t)r.e * D * R + c;
        if constexpr (D == 2) return interp2(__ldg(q), __ldg(q + R), r.k0);
        else return interp3(__ldg(q), __ldg(q + R), __ldg(q + 2 * R), r.k0, r.k1, r.k2);
    }
    __device__ __forceinline__ float cv_at(uint32_t e, uint32_t c) const { return __ldg(cv + (size_t)e * R + c); }
};

constexpr uint32_t kFull = 0xffffffffu;

template <int D, int kBie, int kStrat, bool kUnknown, bool kCV>
__global__ void __launch_bounds__(kBlock, 5) multi_rhs_kernel(SceneView<D> s, WalkParams p, const float *__restrict__ pts,
                                                           BoundaryInput bin, RhsData<D> rd, uint32_t n_points,
                                                           double *__restrict__ sum, double *__restrict__ sumsq,
                                                           unsigned long long *__restrict__ bounces,
                                                           float *__restrict__ per_path) {
    static_assert(!(kUnknown && kCV), "the control variate applies to the domain estimate");
    __shared__ float s_acc[kBlock / 32][32][kMaxRhs];
    __shared__ TapeEntry s_tape[kBlock / 32][32];
    const uint32_t lane = threadIdx.x & 31u;
    float(*acc)[kMaxRhs] = s_acc[threadIdx.x >> 5];
    TapeEntry *tape = s_tape[threadIdx.x >> 5];
    const uint32_t R = rd.R;
    const uint64_t warp = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint64_t n_warps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    const uint32_t span = 32u * p.ppt;
    const uint32_t slabs = (p.n_paths + span - 1u) / span;
    const uint64_t units = (uint64_t)n_points * slabs;
    unsigned long long my_bounces = 0;
    for (uint64_t u = warp; u < units; u += n_warps) {
        const uint32_t pt = (uint32_t)(u / slabs);
        const uint32_t first = (uint32_t)(u % slabs) * span;
        double a_sum[2] = {0.0, 0.0}, a_sq[2] = {0.0, 0.0};
        for (uint32_t sub = 0; sub < p.ppt; sub++) {
            const uint32_t path0 = first + sub * 32u;
            const uint32_t path = path0 + lane;
            const bool active = path < p.n_paths;
#pragma unroll 8
            for (uint32_t j = 0; j < 32; j++) {
                acc[j][lane] = 0.0f;
                acc[j][lane + 32] = 0.0f;
            }
            MultiWalker<D, kBie, kStrat> w(s, p, kUnknown ? kStreamBoundary : kStreamDomain, p.point_offset + pt,
                                           p.path_offset + path);
            BPoint<D> yprev = bp_zero<D>();
            PRef yref{kRefZero, 0.0f, 0.0f, 0.0f};
            PRef y1ref{kRefZero, 0.0f, 0.0f, 0.0f};
            float sdu_v = 0.0f, k0 = 0.0f;
            uint32_t e0 = 0;
            V<D> x = vzero<D>();
            if (active) {
                if constexpr (kUnknown) {
#pragma unroll
                    for (int i = 0; i < D; i++) {
                        yprev.p.v[i] = __ldg(bin.p + (size_t)pt * D + i);
                        yprev.n.v[i] = __ldg(bin.n + (size_t)pt * D + i);
                    }
                    yprev.angle = __ldg(bin.angle + pt);
                    yprev.bv = 0.0f;
                    yprev.type = __ldg(bin.type + pt);
                    yprev.alpha = bin.alpha ? __ldg(bin.alpha + pt) : 0.0f;
                    yref.e = kRefInput;
                } else {
                    // compute_sample_path_contribution_domain (estimator.cuh:154-191): start points y
                    // (unknown term) and y1 (known term), both uniform.
#pragma unroll
                    for (int i = 0; i < D; i++) x.v[i] = __ldg(pts + (size_t)pt * D + i);
                    BPoint<D> y, y1;
                    float ip, ip1;
                    PRef r, r1;
                    sample_uniform_pair_ref<D>(s, w.rng, y, ip, r, y1, ip1, r1);
                    if constexpr (kStrat == kStratUniform) {  // direct sdk: 0 + k0 * (data(y1) + 0)
                        if (y1.type == kDirichlet) k0 = -w.dtc() * ip1 * w.K.dG_dny(y1.p, x, y1.n);
                        else k0 = w.dtc() * ip1 * w.K.G(y1.p, x);
                        y1ref = r1;
                    }
                    sdu_v = w.sdu(x, y, ip);
                    yprev = y;
                    yref = r;
                    e0 = r.e;
                }
            }
            // compute_sample_unknown_boundary (estimator.cuh:232-357), one bounce per step of the warp
            float wgt = 1.0f;
            bool alive = active;
            const uint32_t L = p.path_length;
            for (uint32_t m = 0; m < L; m++) {
                const uint32_t live = __ballot_sync(kFull, alive);
                if (!live) break;
                if (alive) {
                    w.bounces++;
                    if (m == L - 1) wgt = 0.5f * wgt;
                    TapeEntry e;
                    // with a control variate the potential samples are drawn after the walk from the
                    // same stream, so the last transport's draws must still be taken
                    w.bounce(yprev, yref, wgt, e, !kCV && m == L - 1);
                    tape[lane] = e;
                    alive = !(wgt == 0.0f);
                }
                __syncwarp();
                for (uint32_t v = live; v; v &= v - 1u) {
                    const uint32_t j = __ffs(v) - 1u;
                    const TapeEntry e = tape[j];
#pragma unroll
                    for (int h = 0; h < 2; h++) {
                        const uint32_t c = lane + 32u * h;
                        if (c < R) {
                            float T;
                            if constexpr (kStrat == kStratSingleLayer) {
                                T = e.c * (rd.at(e.a, pt, c) + 0.0f);
                            } else {
                                if (e.form == kFormD) {
                                    T = e.k * (rd.at(e.b, pt, c) + 0.0f);
                                } else {
                                    const float sx = rd.at(e.a, pt, c) + 0.0f;
                                    const float sy = rd.at(e.b, pt, c) + 0.0f;
                                    T = e.form == kFormB ? e.c * (sx + e.k * sy) : e.c * (sx - e.k * sy);
                                }
                            }
                            acc[j][c] = acc[j][c] + e.w * T;
                        }
                    }
                }
                __syncwarp();
            }
            my_bounces += w.bounces;
            // path values in place: out = sdk + (mu - cv(y0)) * sdu (domain) or mu (unknown boundary)
            const uint32_t act = __ballot_sync(kFull, active);
            if constexpr (!kUnknown) {
                for (uint32_t j = 0; j < 32u; j++) {
                    if (!((act >> j) & 1u)) continue;
                    const float sdu_j = __shfl_sync(kFull, sdu_v, j);
                    const uint32_t e0j = __shfl_sync(kFull, e0, j);
                    PRef r1j;
                    float k0j = 0.0f;
                    if constexpr (kStrat == kStratUniform) {
                        k0j = __shfl_sync(kFull, k0, j);
                        r1j.e = __shfl_sync(kFull, y1ref.e, j);
                        r1j.k0 = __shfl_sync(kFull, y1ref.k0, j);
                        r1j.k1 = __shfl_sync(kFull, y1ref.k1, j);
                        r1j.k2 = __shfl_sync(kFull, y1ref.k2, j);
                    }
#pragma unroll
                    for (int h = 0; h < 2; h++) {
                        const uint32_t c = lane + 32u * h;
                        if (c < R) {
                            float out0 = 0.0f;
                            if constexpr (kStrat == kStratUniform) out0 = out0 + k0j * (rd.at(r1j, pt, c) + 0.0f);
                            if constexpr (kCV) acc[j][c] = out0 + (acc[j][c] - rd.cv_at(e0j, c)) * sdu_j;
                            else acc[j][c] = out0 + acc[j][c] * sdu_j;
                        }
                    }
                }
                if constexpr (kCV) {
                    // potential of the control variate: n_pot uniform samples per path, after the walk
                    for (uint32_t i = 0; i < rd.n_pot; i++) {
                        if (active) {
                            float ip;
                            PRef r;
                            const BPoint<D> z = sample_uniform_ref<D>(s, w.rng, ip, r);
                            TapeEntry e;
                            e.w = w.sdu(x, z, ip) / (float)rd.n_pot;
                            e.a = r;
                            tape[lane] = e;
                        }
                        __syncwarp();
                        for (uint32_t v = act; v; v &= v - 1u) {
                            const uint32_t j = __ffs(v) - 1u;
                            const float pw = tape[j].w;
                            const uint32_t ez = tape[j].a.e;
#pragma unroll
                            for (int h = 0; h < 2; h++) {
                                const uint32_t c = lane + 32u * h;
                                if (c < R) acc[j][c] = acc[j][c] + pw * rd.cv_at(ez, c);
                            }
                        }
                        __syncwarp();
                    }
                }
            }
            for (uint32_t v = act; v; v &= v - 1u) {
                const uint32_t j = __ffs(v) - 1u;
#pragma unroll
                for (int h = 0; h < 2; h++) {
                    const uint32_t c = lane + 32u * h;
                    if (c < R) {
                        const float out = acc[j][c];
                        if (per_path) per_path[((size_t)pt * p.n_paths + path0 + j) * R + c] = out;
                        const double dv = (double)out;
                        a_sum[h] += dv;
                        a_sq[h] += dv * dv;
                    }
                }
            }
        }
        if (sum) {
#pragma unroll
            for (int h = 0; h < 2; h++) {
                const uint32_t c = lane + 32u * h;
                if (c < R) {
                    atomicAdd(sum + (size_t)pt * R + c, a_sum[h]);
                    if (sumsq) atomicAdd(sumsq + (size_t)pt * R + c, a_sq[h]);
                }
            }
        }
    }
    if (bounces) {
        __syncwarp();
        const unsigned long long b = warp_sum_u64(my_bounces);
        if (lane == 0 && b) atomicAdd(bounces, b);
    }
}

template <int D, int kBie, int kStrat, bool kUnknown, bool kCV>
cudaError_t launch_one(const SceneView<D> &s, const WalkParams &p_in, const float *pts, const BoundaryInput &bin,
                       const RhsData<D> &rd, uint32_t n_points, double *sum, double *sumsq, unsigned long long *bounces,
                       float *per_path, cudaStream_t stream) {
    WalkParams p = p_in;
    p.ppt = choose_ppt(n_points, p.n_paths);
    const uint64_t units = (uint64_t)n_points * ((p.n_paths + 32u * p.ppt - 1u) / (32u * p.ppt));
    auto k = multi_rhs_kernel<D, kBie, kStrat, kUnknown, kCV>;
    k<<<persistent_grid(k, units), kBlock, 0, stream>>>(s, p, pts, bin, rd, n_points, sum, sumsq, bounces, per_path);
    return cudaGetLastError();
}

template <int D>
cudaError_t launch_multi(const SceneView<D> &s, const WalkParams &p, const MultiRhsArgs &a) {
    const RhsData<D> rd{a.rhs_table, a.rhs_input, a.cv_table, a.n_rhs, a.n_potential};
    const bool sl = p.bie == kSingleLayer;
    cudaStream_t st = a.stream;
#define WOB_MRHS_LAUNCH(BIE, STRAT, UNK, CV) \
    launch_one<D, BIE, STRAT, UNK, CV>(s, p, a.points, a.bin, rd, a.n_points, a.sum, a.sumsq, a.bounces, a.per_path, st)
    if (a.unknown) return sl ? WOB_MRHS_LAUNCH(kSingleLayer, kStratSingleLayer, true, false)
                             : WOB_MRHS_LAUNCH(kDirect, kStratUniform, true, false);
    if (a.cv_table) return sl ? WOB_MRHS_LAUNCH(kSingleLayer, kStratSingleLayer, false, true)
                              : WOB_MRHS_LAUNCH(kDirect, kStratUniform, false, true);
    return sl ? WOB_MRHS_LAUNCH(kSingleLayer, kStratSingleLayer, false, false)
              : WOB_MRHS_LAUNCH(kDirect, kStratUniform, false, false);
#undef WOB_MRHS_LAUNCH
}

}  // namespace mrhs
}  // namespace wobgb
