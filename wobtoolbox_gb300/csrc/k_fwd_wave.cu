// Forward single-layer Neumann walk in 3D (estimator.cuh:405-454, the exterior Neumann workload's
// estimator) as a split-phase wavefront: the paths' line queries are taken out of the walk and run
// by a kernel that does nothing else.
//
// In the lockstep kernel (kernels.cuh) a warp's 32 paths run their bounces together, and each
// bounce waits for the longest of the 32 line queries: the 3D query's length varies several-fold
// with the line (grazing lines cross many boxes), so most lanes idle (6 of 32 lanes active per
// instruction, measured). Here a chunk of paths advances in phases, each a kernel over the chunk:
//   start    -- one thread per path: the source samples, the first bounce's terms and the first
//               line query's direction;
//   trace    -- persistent: every lane takes the next pending query (one atomic per warp for all
//               lanes that need one) as soon as its previous query has ended, so a lane never
//               waits for another lane's query; the traversal is line_query3's (shared-memory
//               stack columns, first kept child from a register, postponed leaves), optionally on
//               64-byte compressed nodes built per solve, and the hit is chosen where the hits are
//               (line_hit_choice, the path's own next draw);
//   consume  -- one thread per path: the hit's point, the transport weight, the next bounce's terms
//               and the next direction (repeated path_length - 1 times with trace);
//   reduce   -- one warp per point: FP64 sums and squares over its paths.
// Every path runs the operations of Walker's forward branch in the same order on its own Philox
// stream (its position, PathRng::drawn, is kept between phases), so every path value is
// bit-identical to the lockstep kernel's and the CPU oracle's; only the order of the FP64 sums
// over a point's paths differs. Path state lives in HBM between phases (about 84 bytes a path,
// structure of arrays, coalesced), in chunks of whole points.
#include "kernels.cuh"

namespace wobgb {

namespace {

constexpr uint32_t kFull = 0xffffffffu;
constexpr int kYWords = 10;  // BPoint<3>: p (3), n (3), angle, bv, type (bits), alpha

struct WaveArgs {
    const float *pts;
    uint32_t pt0, n_pts;    // the chunk's points
    uint32_t n;             // slots: n_pts x n_paths, slot j = (pt0 + j / n_paths, path j % n_paths)
    uint32_t *draws;        // [n] uniforms drawn on the path's stream
    float *y;               // [kYWords][n] the current boundary point
    float *wt;              // [n] transport weight
    float *out;             // [4][n] u and grad u of the path so far
    float *dir;             // [3][n] pending line query's direction (origin: y.p)
    uint32_t *hit;          // [n] the chosen element of the finished query
    uint32_t *nhit;         // [n] min(hits, 64); 0: no hit
    uint32_t *counter;      // trace: next slot to hand out
};

using FwdWalker = Walker<3, kSingleLayer, kStratFwdSlNeumann, false>;

__device__ __forceinline__ void store_y(const WaveArgs &a, uint32_t j, const BPoint<3> &y) {
    const float w[kYWords] = {y.p.v[0], y.p.v[1], y.p.v[2], y.n.v[0], y.n.v[1], y.n.v[2],
                              y.angle, y.bv, __int_as_float(y.type), y.alpha};
#pragma unroll
    for (int k = 0; k < kYWords; k++) a.y[(size_t)k * a.n + j] = w[k];
}
__device__ __forceinline__ BPoint<3> load_y(const WaveArgs &a, uint32_t j) {
    float w[kYWords];
#pragma unroll
    for (int k = 0; k < kYWords; k++) w[k] = a.y[(size_t)k * a.n + j];
    BPoint<3> y;
    y.p.v[0] = w[0]; y.p.v[1] = w[1]; y.p.v[2] = w[2];
    y.n.v[0] = w[3]; y.n.v[1] = w[4]; y.n.v[2] = w[5];
    y.angle = w[6];
    y.bv = w[7];
    y.type = __float_as_int(w[8]);
    y.alpha = w[9];
    return y;
}

__device__ __forceinline__ void slot_point(const WalkParams &p, const WaveArgs &a, uint32_t j, uint32_t &pt,
                                           uint32_t &path) {
    pt = a.pt0 + j / p.n_paths;
    path = j % p.n_paths;
}

// The m-th bounce's terms: out += w sdu(x, y), w gdu(x, y), the weight halved on the last bounce.
__device__ __forceinline__ void bounce_terms(FwdWalker &w, const V<3> &x, const BPoint<3> &y, float &wt, uint32_t m,
                                             uint32_t L, float out[4]) {
    w.bounces++;
    if (m == L - 1) wt = wt * 0.5f;
    out[0] = out[0] + wt * w.sdu(x, y, 1.0f);
    const V<3> gu = w.gdu(x, y, 1.0f);
#pragma unroll
    for (int i = 0; i < 3; i++) out[1 + i] = out[1 + i] + wt * gu.v[i];
}

__device__ __forceinline__ V<3> load_x(const WaveArgs &a, uint32_t pt) {
    V<3> x;
#pragma unroll
    for (int i = 0; i < 3; i++) x.v[i] = __ldg(a.pts + (size_t)pt * 3 + i);
    return x;
}

__global__ void __launch_bounds__(kWalkBlock) wave_start_kernel(SceneView<3> s, WalkParams p, WaveArgs a) {
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= a.n) return;
    uint32_t pt, path;
    slot_point(p, a, j, pt, path);
    FwdWalker w(s, p, kStreamDomain, p.point_offset + pt, p.path_offset + path);
    const V<3> x = load_x(a, pt);
    // Walker::domain, forward branch: the known term's sample, then the transported source
    float out[4], ip, ip2;
    BPoint<3> y = sample_uniform<3>(s, w.rng, ip);
    out[0] = w.sdk(x, y, ip);
    const V<3> g = w.gdk(x, y, ip);
#pragma unroll
    for (int i = 0; i < 3; i++) out[1 + i] = g.v[i];
    y = sample_boundary_value<3>(s, w.rng, ip);
    const BPoint<3> y2 = sample_uniform<3>(s, w.rng, ip2);
    float wt = ip * w.fbk(y, y2, ip2);
    const uint32_t L = p.path_length;
    bounce_terms(w, x, y, wt, 0, L, out);
    if (L > 1) {
        const V<3> d = line_sample_direction<3>(w.rng);
#pragma unroll
        for (int i = 0; i < 3; i++) a.dir[(size_t)i * a.n + j] = d.v[i];
    }
    store_y(a, j, y);
    a.wt[j] = wt;
#pragma unroll
    for (int c = 0; c < 4; c++) a.out[(size_t)c * a.n + j] = out[c];
    a.draws[j] = w.rng.drawn();
}

// Compressed BVH nodes for the trace phase: 64 bytes instead of 128 (two 32-byte sectors a visit
// instead of four). Each child's box is stored as 8-bit offsets on a power-of-two grid over the
// node's own box: words 0-2 the node box's lower corner o (float), word 3 the grid's biased
// exponents per axis (byte a), words 4-7 the children, words 8-13 the quantized bounds (word 8 + a:
// lower bound on axis a, byte k for child k; word 11 + a: upper bounds), words 14-15 zero. Lower
// bounds are rounded down and upper bounds up (in double), so every decoded box contains its
// child's padded box up to one float rounding of o + q 2^e -- far inside the boxes' 1e-5 padding:
// the box test stays conservative and the hits (decided by the exact triangle test) are unchanged.
constexpr int kQNodeWords = 16;

__global__ void compress_nodes_kernel(const float4 *__restrict__ soa, uint32_t n_nodes, uint32_t *__restrict__ out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_nodes) return;
    const float *q = reinterpret_cast<const float *>(soa + 8 * (size_t)i);
    const uint32_t *c = reinterpret_cast<const uint32_t *>(q + 24);
    uint32_t w[kQNodeWords] = {};
    double lo[3], ext[3];
    for (int a = 0; a < 3; a++) {
        double mn = 1e300, mx = -1e300;
        for (int k = 0; k < 4; k++) {
            if (c[k] == kChildEmptyD) continue;
            mn = fmin(mn, (double)q[4 * a + k]);
            mx = fmax(mx, (double)q[12 + 4 * a + k]);
        }
        if (mn > mx) mn = mx = 0.0;
        const float o = (float)mn <= mn ? (float)mn : nextafterf((float)mn, -INFINITY);  // o <= every lower bound
        lo[a] = (double)o;
        ext[a] = mx - lo[a];
        int e = 0;
        frexp(ext[a] / 255.0, &e);  // 2^e > ext / 255: 255 steps of 2^e cover the box
        if (ext[a] <= 0.0) e = -126;
        e = e < -126 ? -126 : (e > 127 ? 127 : e);
        w[a] = __float_as_uint(o);
        w[3] |= (uint32_t)(e + 127) << (8 * a);
        const double step = ldexp(1.0, e);
        for (int k = 0; k < 4; k++) {
            double ql = 0.0, qh = 0.0;
            if (c[k] != kChildEmptyD) {
                ql = floor(((double)q[4 * a + k] - lo[a]) / step);
                qh = ceil(((double)q[12 + 4 * a + k] - lo[a]) / step);
            }
            ql = fmin(fmax(ql, 0.0), 255.0);
            qh = fmin(fmax(qh, 0.0), 255.0);
            w[8 + a] |= (uint32_t)ql << (8 * k);
            w[11 + a] |= (uint32_t)qh << (8 * k);
        }
    }
    for (int k = 0; k < 4; k++) w[4 + k] = c[k];
    uint4 *dst = reinterpret_cast<uint4 *>(out + (size_t)i * kQNodeWords);
    for (int v = 0; v < 4; v++) dst[v] = make_uint4(w[4 * v], w[4 * v + 1], w[4 * v + 2], w[4 * v + 3]);
}

// The slab test against a compressed node's four children. With the node's corner o and grid step
// s = 2^e per axis, a child bound o + q s lies on the line at t = q (s r) + (o r - O r): s r is exact
// (a power of two times r), o r - O r one FMA per axis and node, and each bound then one FMA. q is
// formed exactly by a byte permute into the float 2^23 + q and one subtraction, which keeps the
// conversion off the special-function pipe. The t's rounding is of the order of the uncompressed
// test's, far inside the boxes' padding.
__device__ __forceinline__ float qbyte(uint32_t word, uint32_t k) {
    return __uint_as_float(__byte_perm(word, 0x4B000000u, 0x7540u + k)) - 8388608.0f;
}
__device__ __forceinline__ uint32_t qnode_hits(const uint32_t *__restrict__ qn, uint32_t node, const LineSlab3 &L,
                                               uint4 &child) {
    const float4 *p = reinterpret_cast<const float4 *>(qn + (size_t)node * kQNodeWords);
    const F8 r0 = ldg8(p), r1 = ldg8(p + 2);
    const float o[3] = {r0.a.x, r0.a.y, r0.a.z};
    const uint32_t ex = __float_as_uint(r0.a.w);
    child = make_uint4(__float_as_uint(r0.b.x), __float_as_uint(r0.b.y), __float_as_uint(r0.b.z),
                       __float_as_uint(r0.b.w));
    const uint32_t qlo[3] = {__float_as_uint(r1.a.x), __float_as_uint(r1.a.y), __float_as_uint(r1.a.z)};
    const uint32_t qhi[3] = {__float_as_uint(r1.a.w), __float_as_uint(r1.b.x), __float_as_uint(r1.b.y)};
    float A[3], B[3];
#pragma unroll
    for (int a = 0; a < 3; a++) {
        A[a] = __uint_as_float(((ex >> (8 * a)) & 0xFFu) << 23) * L.r[a];
        B[a] = __fmaf_rn(o[a], L.r[a], L.nor[a]);
    }
    uint32_t mask = 0;
#pragma unroll
    for (int k = 0; k < 4; k++) {
        float tl[3], th[3];
#pragma unroll
        for (int a = 0; a < 3; a++) {
            tl[a] = __fmaf_rn(qbyte(qlo[a], (uint32_t)k), A[a], B[a]);
            th[a] = __fmaf_rn(qbyte(qhi[a], (uint32_t)k), A[a], B[a]);
        }
        const float tn = fmax3f(fminf(tl[0], th[0]), fminf(tl[1], th[1]), fminf(tl[2], th[2]));
        const float tf = fmin3f(fmaxf(tl[0], th[0]), fmaxf(tl[1], th[1]), fmaxf(tl[2], th[2]));
        if (tn <= tf) mask |= 1u << k;
    }
    return mask;
}

// The trace phase. kLeaves: leaves a lane holds before testing them (line_query3's kLeafBatch);
// kQuant: node visits read the compressed nodes (qnodes) instead of the scene's.
template <int kMinB, int kLeaves, bool kQuant>
__global__ void __launch_bounds__(kWalkBlock, kMinB) wave_trace_kernel(SceneView<3> s, WalkParams p, WaveArgs a,
                                                                      const uint32_t *__restrict__ qnodes) {
    static_assert(kLeaves <= kLeafBatch, "leaf columns hold kLeafBatch entries");
    const uint32_t lane = threadIdx.x & 31u;
    uint32_t *const my_stack = stack_column();
    uint32_t *const my_leaf = leaf_column();
    uint32_t spill[kStackSize - kSharedStack];
    uint32_t hits[kHitBuffer];
    LineSlab3 L;
    V<3> o, d;
    uint32_t j = 0, code = 0, steps = 0, count = 0;
    int sp = 0;
    bool busy = false, fetch = true;
    while (true) {
        // lanes without a query take the next slots: one atomic for the warp
        const uint32_t need = __ballot_sync(kFull, fetch);
        if (need) {
            const int leader = __ffs(need) - 1;
            uint32_t base = 0;
            if ((int)lane == leader) base = atomicAdd(a.counter, (uint32_t)__popc(need));
            base = __shfl_sync(kFull, base, leader);
            if (fetch) {
                j = base + (uint32_t)__popc(need & ((1u << lane) - 1u));
                fetch = false;
                busy = j < a.n;
                if (busy) {
#pragma unroll
                    for (int i = 0; i < 3; i++) {
                        o.v[i] = a.y[(size_t)i * a.n + j];
                        d.v[i] = a.dir[(size_t)i * a.n + j];
                    }
                    L = line_slab3(o, d);
                    code = 0u;  // root node
                    sp = 0;
                    steps = 0;
                    count = 0;
                }
            }
        }
        if (!__any_sync(kFull, busy)) break;
        if (!busy) continue;
        // one round of line_query3: nodes until kLeaves leaves are held or the stack is empty,
        // then the held leaves in the order they were met
        int nl = 0;
        bool live = true;
        while (nl < kLeaves) {
            if (++steps > s.traversal_limit) {
                atomicOr(s.err, kErrTraversalLimit);
                live = false;
                break;
            }
            if (code & 0x80000000u) {
                my_leaf[nl * kWalkBlock] = code;
                nl++;
            } else {
                uint4 ch;
                uint32_t keep = kQuant ? qnode_hits(qnodes, code, L, ch) : node_hits(s, code, L, ch);
                const uint32_t cs[4] = {ch.x, ch.y, ch.z, ch.w};
#pragma unroll
                for (int k = 0; k < 4; k++)
                    if (cs[k] == kChildEmptyD) keep &= ~(1u << k);
                if (keep) {
                    if (sp + 3 > (int)kStackSize) {
                        atomicOr(s.err, kErrStackOverflow);
                        live = false;
                        break;
                    }
                    const uint32_t first = (uint32_t)(__ffs(keep) - 1);
#pragma unroll
                    for (int k = 3; k >= 1; k--)
                        if ((uint32_t)k > first && ((keep >> k) & 1u)) {
                            if (sp < kSharedStack) my_stack[sp * kWalkBlock] = cs[k];
                            else spill[sp - kSharedStack] = cs[k];
                            sp++;
                        }
                    code = cs[first];
                    continue;
                }
            }
            if (sp == 0) {
                live = false;
                break;
            }
            sp--;
            code = sp < kSharedStack ? my_stack[sp * kWalkBlock] : spill[sp - kSharedStack];
        }
        for (int l = 0; l < nl; l++) count = leaf_hits<3>(s, my_leaf[l * kWalkBlock], o, d, hits, count);
        if (!live) {
            // the query is complete: choose the hit with the path's next draw
            uint32_t pt, path;
            slot_point(p, a, j, pt, path);
            PathRng rng(p.seed, kStreamDomain, p.point_offset + pt, p.path_offset + path);
            rng.seek(a.draws[j]);
            uint32_t m = count;
            a.hit[j] = line_hit_choice(rng, hits, m);
            a.nhit[j] = m;
            busy = false;
            fetch = true;
        }
    }
}

// Bounce m (1 <= m < L) of every path: the chosen hit's point, the transport, the bounce's terms
// and, below the last bounce, the next direction.
__global__ void __launch_bounds__(kWalkBlock) wave_consume_kernel(SceneView<3> s, WalkParams p, WaveArgs a,
                                                                  uint32_t m) {
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= a.n) return;
    uint32_t pt, path;
    slot_point(p, a, j, pt, path);
    FwdWalker w(s, p, kStreamDomain, p.point_offset + pt, p.path_offset + path);
    w.rng.seek(a.draws[j]);
    const V<3> x = load_x(a, pt);
    BPoint<3> y_prev = load_y(a, j);
    V<3> dir;
#pragma unroll
    for (int i = 0; i < 3; i++) dir.v[i] = a.dir[(size_t)i * a.n + j];
    const uint32_t nh = a.nhit[j];
    if (nh) (void)w.rng.uniform();  // the hit choice's draw, taken in the trace phase
    BPoint<3> y = line_hit_point<3>(s, a.hit[j], nh, y_prev.p, dir);
    const float ip = line_sample_inv_pdf<3>(y, y_prev.p, nh);
    float wt = a.wt[j];
    wt = w.fbu(y, y_prev, ip, false) * wt;
    float out[4];
#pragma unroll
    for (int c = 0; c < 4; c++) out[c] = a.out[(size_t)c * a.n + j];
    const uint32_t L = p.path_length;
    bounce_terms(w, x, y, wt, m, L, out);
    if (m + 1 < L) {
        const V<3> d = line_sample_direction<3>(w.rng);
#pragma unroll
        for (int i = 0; i < 3; i++) a.dir[(size_t)i * a.n + j] = d.v[i];
    }
    store_y(a, j, y);
    a.wt[j] = wt;
#pragma unroll
    for (int c = 0; c < 4; c++) a.out[(size_t)c * a.n + j] = out[c];
    a.draws[j] = w.rng.drawn();
}

// One warp per point of the chunk: FP64 sums and squares over its paths, per-path records.
__global__ void __launch_bounds__(kWalkBlock) wave_reduce_kernel(WalkParams p, WaveArgs a, double *__restrict__ sum,
                                                                 double *__restrict__ sumsq,
                                                                 unsigned long long *__restrict__ bounces,
                                                                 float *__restrict__ per_path) {
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t q = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (blockIdx.x == 0 && threadIdx.x == 0 && bounces)
        atomicAdd(bounces, (unsigned long long)a.n * p.path_length);
    if (q >= a.n_pts) return;
    const uint32_t pt = a.pt0 + q;
    double acc[8];
#pragma unroll
    for (int c = 0; c < 8; c++) acc[c] = 0.0;
    for (uint32_t path = lane; path < p.n_paths; path += 32u) {
        const uint32_t j = q * p.n_paths + path;
#pragma unroll
        for (int c = 0; c < 4; c++) {
            const float v = a.out[(size_t)c * a.n + j];
            if (per_path) per_path[((size_t)pt * p.n_paths + path) * 4 + c] = v;
            const double dv = (double)v;
            acc[c] += dv;
            acc[4 + c] += dv * dv;
        }
    }
    if (!sum) return;
#pragma unroll
    for (int c = 0; c < 4; c++) {
        const double sv = warp_sum(acc[c]);
        const double qv = warp_sum(acc[4 + c]);
        if (lane == 0) {
            atomicAdd(sum + (size_t)pt * 4 + c, sv);
            if (sumsq) atomicAdd(sumsq + (size_t)pt * 4 + c, qv);
        }
    }
}

template <int kMinB, int kLeaves, bool kQuant>
cudaError_t trace(const SceneView<3> &s, const WalkParams &p, const WaveArgs &a, const uint32_t *qnodes,
                  cudaStream_t stream) {
    auto k = wave_trace_kernel<kMinB, kLeaves, kQuant>;
    int per_sm = 0, dev = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, kWalkBlock, 0);
    if (e != cudaSuccess) return e;
    const uint64_t need = ((uint64_t)a.n + kWalkBlock - 1) / kWalkBlock;
    const uint64_t grid = std::min<uint64_t>(need, (uint64_t)std::max(1, per_sm) * (uint64_t)sms);
    if ((e = cudaMemsetAsync(a.counter, 0, sizeof(uint32_t), stream)) != cudaSuccess) return e;
    k<<<(unsigned)grid, kWalkBlock, 0, stream>>>(s, p, a, qnodes);
    return cudaGetLastError();
}

}  // namespace

cudaError_t launch_fwd_wave_3d(const SceneView<3> &s, const WalkParams &p, const float *pts, uint32_t n_points,
                               double *sum, double *sumsq, unsigned long long *bounces, float *per_path, int shape,
                               uint32_t max_slots, cudaStream_t stream) {
    if (n_points == 0 || p.n_paths == 0) return cudaSuccess;
    const uint32_t chunk_pts = std::max<uint32_t>(1u, max_slots / p.n_paths);
    const uint64_t slots = (uint64_t)std::min(chunk_pts, n_points) * p.n_paths;
    if (slots > 0xFFFFFFFFull / 2) return cudaErrorInvalidValue;
    const size_t n = (size_t)slots;
    const bool quant = shape == 3;
    const size_t words = n * (1 + kYWords + 1 + 4 + 3 + 2) + 1;
    const size_t q_off = (words * 4 + 255) / 256 * 256;  // bytes; the compressed nodes 256-byte aligned
    const size_t bytes = q_off + (quant ? (size_t)s.n_nodes * kQNodeWords * 4 : 0);
    void *buf = nullptr;
    cudaError_t e = cudaMallocAsync(&buf, bytes, stream);
    if (e != cudaSuccess) return e;
    uint32_t *qnodes = quant ? (uint32_t *)((char *)buf + q_off) : nullptr;
    if (quant && s.n_nodes) {
        compress_nodes_kernel<<<(s.n_nodes + 127) / 128, 128, 0, stream>>>(s.nodes, s.n_nodes, qnodes);
        e = cudaGetLastError();
    }
    WaveArgs a{};
    a.pts = pts;
    uint32_t *w = (uint32_t *)buf;
    a.draws = w;
    a.y = (float *)(w + n);
    a.wt = (float *)(w + n * (1 + kYWords));
    a.out = (float *)(w + n * (2 + kYWords));
    a.dir = (float *)(w + n * (6 + kYWords));
    a.hit = w + n * (9 + kYWords);
    a.nhit = w + n * (10 + kYWords);
    a.counter = w + n * (11 + kYWords);
    for (uint32_t pt0 = 0; pt0 < n_points && e == cudaSuccess; pt0 += chunk_pts) {
        a.pt0 = pt0;
        a.n_pts = std::min(chunk_pts, n_points - pt0);
        a.n = a.n_pts * p.n_paths;
        const unsigned blocks = (a.n + kWalkBlock - 1) / kWalkBlock;
        wave_start_kernel<<<blocks, kWalkBlock, 0, stream>>>(s, p, a);
        e = cudaGetLastError();
        for (uint32_t m = 1; m < p.path_length && e == cudaSuccess; m++) {
            switch (shape) {
            case 1: e = trace<8, 8, false>(s, p, a, nullptr, stream); break;
            case 2: e = trace<6, 8, false>(s, p, a, nullptr, stream); break;
            default: e = trace<6, 8, true>(s, p, a, qnodes, stream); break;
            }
            if (e != cudaSuccess) break;
            wave_consume_kernel<<<blocks, kWalkBlock, 0, stream>>>(s, p, a, m);
            e = cudaGetLastError();
        }
        if (e != cudaSuccess) break;
        const unsigned rblocks = (a.n_pts * 32u + kWalkBlock - 1) / kWalkBlock;
        wave_reduce_kernel<<<rblocks, kWalkBlock, 0, stream>>>(p, a, sum, sumsq, bounces, per_path);
        e = cudaGetLastError();
    }
    const cudaError_t f = cudaFreeAsync(buf, stream);
    return e != cudaSuccess ? e : f;
}

}  // namespace wobgb
