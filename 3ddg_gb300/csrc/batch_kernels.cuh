// Batched form: many independent problems of uneven element counts and
// orders advanced together, FP32 fields/fluxes/stages with the
// Kahan-compensated update.
//
// Each problem keeps its own device buffers and a device descriptor
// (BatchProblem) with its FP32 operators, RK weights, time and source state,
// so problems can join and leave (the serving form) without touching the
// others.  Problems of one order that share one operator form a group; per
// RK stage each group gets two launches of a persistent kernel of its order
// (batch_stage_kernel<K>, K = N + 1 <= 6) that pull tiles (problem, first
// element, element count) from an atomic counter: the LDG gradient of every
// tile, then the stage update of every tile, with EPB(K) elements per pass of
// a CTA of bthreads_of(K) threads; the number of passes per tile (tile size) is chosen per
// order by the autotuner.  Groups run as parallel branches of the step.  The
// arithmetic per element is the one of incr_stage_kernel /
// ldg_gradient_kernel (dg_kernels.cuh) with 1/w_a applied after the line
// sums, so one descriptor serves all three stages and the group's operator
// rows (kernel parameters) do not depend on the axis.  Face nodes are decoded
// arithmetically (FaceNodeArith): the table lookup the single-problem kernels
// use measured 2 % slower here (115.1 vs 117.3 G on config 4).
#pragma once


#include "batch_types.h"
#include "dg_kernels.cuh"

namespace dg {

// Threads per CTA of order K: 256, except one element's 224 node slots at
// K = 6, where a 256-thread CTA would carry an idle warp that holds registers
// (and resident-CTA slots) without work in the node phases.
__host__ __device__ constexpr int bthreads_of(int K) { return K == 6 ? npt_of(6) : BATCH_THREADS; }
__host__ __device__ constexpr int bepb_of(int K) { return bthreads_of(K) / npt_of(K); }

__device__ __forceinline__ void batch_exterior(const BatchProblem& P, int face, int stage, float& ro, float& uo)
{
    if (face == P.src_face) {
        const float p = P.src_p[stage];
        ro = p * P.inv_c2;
        uo = ((face & 1) ? -p : p) * P.inv_z;
    } else {
        ro = 0.f;
        uo = 0.f;
    }
}

template <int K>
__device__ __forceinline__ float batch_in(const BatchProblem& P, const float* ub, const float* inc, int f, size_t off)
{
    float v = __ldg(ub + (size_t)f * P.fs + off);
    if (inc) v += __ldg(inc + (size_t)f * P.fs + off);
    return v;
}

// Face-table codes of the face nodes this thread evaluates in the pass whose
// first element is c0 (0 where it has none).
template <int K, int R>
__device__ __forceinline__ void batch_codes(const BatchProblem& P, const BatchTile& T, int c0, int slot, int n,
                                            int code[R])
{
    constexpr int NPT = npt_of(K), EPB = bepb_of(K), NF = 6 * K * K;
    const int e = c0 + slot;
    const bool live = slot < EPB && e < T.e0 + T.count;
#pragma unroll
    for (int r = 0; r < R; r++) {
        const int t = n + r * NPT;
        code[r] = 0;
        if (live && t < NF) {
            const FaceNodeArith<K> F(t);
            code[r] = __ldg(P.nbr + (size_t)e * 6 + 2 * F.a + F.side);
        }
    }
}

template <int K>
__device__ __forceinline__ float batch_sigma(const BatchProblem& P, const BatchTile& T, int c0, int slot, int n)
{
    constexpr int NPT = npt_of(K), EPB = bepb_of(K), K3 = K * K * K;
    const int e = c0 + slot;
    return (slot < EPB && e < T.e0 + T.count && n < K3) ? __ldg(P.sigma + e) : 0.f;
    (void)NPT;
}

// Line task of this thread in a pass of the gradient phase: element slot ls,
// axis a, line t (false: no task).  K = 5: one warp per axis of each element
// slot; K = 6: the element's 108 lines over its first 4 warps; K <= 4: the
// CTA's threads over (slot, axis, line).
template <int K>
__device__ __forceinline__ bool batch_line_task(int slot, int n, int& ls, int& a, int& t)
{
    constexpr int K2 = K * K, WPA = (K2 + 31) / 32, EPB = bepb_of(K);
    if constexpr (K >= 6) {
        a = n / K2;
        t = n % K2;
        ls = slot;
    } else if constexpr (K == 5) {
        const int w = n / 32;
        a = w / WPA;
        t = (w % WPA) * 32 + n % 32;
        ls = slot;
    } else {
        ls = threadIdx.x / (3 * K2);
        a = (threadIdx.x / K2) % 3;
        t = threadIdx.x % K2;
    }
    return ls < EPB && a < 3 && t < K2;
}

// Face-table codes of the two ends of the owner's line (element c0 + ls).
template <int K>
__device__ __forceinline__ void batch_end_codes(const BatchProblem& P, const BatchTile& T, int c0, bool task, int ls,
                                                int a, int code[2])
{
    const int e = c0 + ls;
    const bool live = task && e < T.e0 + T.count;
    code[0] = live ? __ldg(P.nbr + (size_t)e * 6 + 2 * a) : 0;
    code[1] = live ? __ldg(P.nbr + (size_t)e * 6 + 2 * a + 1) : 0;
}

// Shared memory of the gradient phase, per element slot: drho of every node,
// double-buffered by pass parity.
template <int K>
struct BatchGradSmem {
    float r[2][npt_of(K)];
};

// The gradient phase of one tile.  Each line owner loads the neighbour
// values at its line's two ends, forms the two central face fluxes itself
// and stores its line's results (every value of the gradient has one owner),
// so a pass has one barrier: with drho double-buffered, a pass's writes go
// to the buffer the pass before last read, which every owner finished before
// the previous pass's barrier.  The owners' face-table codes of each pass
// are loaded during the pass before.
template <int K>
__device__ void batch_grad_tile(const BatchProblem& P, const BatchOps& ops, const BatchTile& T, int stage,
                                unsigned char* smraw)
{
    constexpr int K2 = K * K, K3 = K * K * K, NPT = npt_of(K), EPB = bepb_of(K);
    BatchGradSmem<K>* SM = reinterpret_cast<BatchGradSmem<K>*>(smraw);
    const int slot = threadIdx.x / NPT, n = threadIdx.x % NPT;
    const float* ub = P.u[P.cur];
    const float* inc = stage == 0 ? nullptr : P.d[stage - 1];
    int ls = 0, a = 0, t = 0;
    const bool task = batch_line_task<K>(slot, n, ls, a, t);
    const int st = axis_stride<K>(a < 3 ? a : 0);
    const int b0 = a == 0 ? t : (a == 1 ? (t % K) * K2 + (t / K) : t * K);
    int code_next[2];
    batch_end_codes<K>(P, T, T.e0, task, ls, a, code_next);
    int buf = 0;
    for (int c0 = T.e0; c0 < T.e0 + T.count; c0 += EPB, buf ^= 1) {
        const int e = c0 + slot;
        const bool act = slot < EPB && e < T.e0 + T.count && n < K3;
        const bool owner = task && c0 + ls < T.e0 + T.count;
        const int code[2] = {code_next[0], code_next[1]};
        batch_end_codes<K>(P, T, c0 + EPB, task, ls, a, code_next);
        // every other global load is issued before the first use
        float rho = 0.f;
        if (act) rho = batch_in<K>(P, ub, inc, 0, (size_t)e * P.np + n);
        float ro[2] = {0.f, 0.f};
        if (owner) {
#pragma unroll
            for (int side = 0; side < 2; side++) {
                if (code[side] >= 0) {
                    const size_t o2 = (size_t)code[side] * P.np + b0 + (side ? 0 : (K - 1) * st);
                    ro[side] = batch_in<K>(P, ub, inc, 0, o2);
                } else {
                    float uo;
                    batch_exterior(P, -1 - code[side], stage, ro[side], uo);
                }
            }
        }
        if (slot < EPB) SM[slot].r[buf][n] = rho;
        __syncthreads();
        if (owner) {
            const float* r = SM[ls].r[buf];
            float* q = P.q + (size_t)a * P.fs + (size_t)(c0 + ls) * P.np;
            float v[K];
#pragma unroll
            for (int j = 0; j < K; j++) v[j] = r[b0 + j * st];
            const float f0 = 0.5f * (ro[0] + v[0]), fN = -0.5f * (ro[1] + v[K - 1]);
            const float gs = P.gscale[a];
#pragma unroll
            for (int i = 0; i < K; i++) {
                const float* row = ops.rows[i];  // constant-bank operands
                float s2 = row[K] * f0;
                s2 += row[K + 1] * fN;
#pragma unroll
                for (int j = 0; j < K; j++) s2 += row[j] * v[j];
                q[b0 + i * st] = gs * s2;
            }
        }
    }
}

template <int K>
__device__ void batch_stage_tile(const BatchProblem& P, const BatchOps& ops, const BatchTile& T, int stage,
                                 unsigned char* smraw)
{
    constexpr int K2 = K * K, K3 = K * K * K, NPT = npt_of(K), EPB = bepb_of(K), NF = 6 * K2;
    constexpr int R = (NF + NPT - 1) / NPT;
    PlainSmem<float, K>* SM = reinterpret_cast<PlainSmem<float, K>*>(smraw);
    const int slot = threadIdx.x / NPT, n = threadIdx.x % NPT;
    const float* ub = P.u[P.cur];
    const float* inc = stage == 0 ? nullptr : P.d[stage - 1];
    const bool final_stage = stage == 2;
    float* dout = final_stage ? P.u[P.cur ^ 1] : P.d[stage];
    const float ca = P.ca[stage], cb = P.cb[stage], eps = final_stage ? P.eps : 0.f;
    // The face-table codes and sigma of each pass are loaded during the pass
    // before, so a pass's neighbour loads wait on one memory latency instead
    // of two chained ones.
    int code_next[R];
    batch_codes<K, R>(P, T, T.e0, slot, n, code_next);
    float sig_next = batch_sigma<K>(P, T, T.e0, slot, n);
    for (int c0 = T.e0; c0 < T.e0 + T.count; c0 += EPB) {
        const int e = c0 + slot;
        const bool live = slot < EPB && e < T.e0 + T.count;
        const bool act = live && n < K3;
        PlainSmem<float, K>& S = SM[slot < EPB ? slot : 0];
        const size_t off = (size_t)e * P.np + n;
        int code[R];
#pragma unroll
        for (int r = 0; r < R; r++) code[r] = code_next[r];
        const float sig = sig_next;
        batch_codes<K, R>(P, T, c0 + EPB, slot, n, code_next);
        sig_next = batch_sigma<K>(P, T, c0 + EPB, slot, n);
        // Every other global load before the first use (the kernel waits on
        // memory latency): the own u, d, gradient and compensation, then the
        // neighbour values of the densely assigned face nodes (see
        // stage_kernel).
        float ubv[4] = {0.f, 0.f, 0.f, 0.f}, dv[4] = {0.f, 0.f, 0.f, 0.f}, cmp[4] = {0.f, 0.f, 0.f, 0.f};
        float q[3] = {0.f, 0.f, 0.f};
        if (act) {
#pragma unroll
            for (int f = 0; f < 4; f++) {
                ubv[f] = __ldg(ub + (size_t)f * P.fs + off);
                if (inc) dv[f] = __ldg(inc + (size_t)f * P.fs + off);
                if (final_stage) cmp[f] = P.comp[(size_t)f * P.fs + off];
            }
#pragma unroll
            for (int a = 0; a < 3; a++) q[a] = __ldg(P.q + (size_t)a * P.fs + off);
        }
        float ro[R], uo[R], qo[R];
#pragma unroll
        for (int r = 0; r < R; r++) {
            ro[r] = uo[r] = qo[r] = 0.f;
            const int t = n + r * NPT;
            if (!live || t >= NF) continue;
            const FaceNodeArith<K> F(t);
            if (code[r] >= 0) {
                const size_t o2 = (size_t)code[r] * P.np + F.nn;
                ro[r] = batch_in<K>(P, ub, inc, 0, o2);
                uo[r] = batch_in<K>(P, ub, inc, 1 + F.a, o2);
                qo[r] = __ldg(P.q + (size_t)F.a * P.fs + o2);
            } else {
                batch_exterior(P, -1 - code[r], stage, ro[r], uo[r]);
            }
        }
        const float rho = ubv[0] + dv[0];
        const float u[3] = {ubv[1] + dv[1], ubv[2] + dv[2], ubv[3] + dv[3]};
        const float fmom = momentum_flux(rho, P.k1, P.k2);
        float fmass[3];
#pragma unroll
        for (int a = 0; a < 3; a++) fmass[a] = mass_flux(u[a], rho, P.r0, P.linear_mass);
        if (slot < EPB) {
#pragma unroll
            for (int a = 0; a < 3; a++) {
                S.f[a][n] = make_float2(fmom, fmass[a] + q[a]);
                S.m[a][n] = fmass[a];
                S.q[a][n] = q[a];
            }
        }
        __syncthreads();
#pragma unroll
        for (int r = 0; r < R; r++) {
            const int t = n + r * NPT;
            if (!live || t >= NF) continue;
            const FaceNodeArith<K> F(t);
            const float fm_s = S.f[F.a][F.nf].x, fa_s = S.m[F.a][F.nf];
            const float fmo = momentum_flux(ro[r], P.k1, P.k2);
            const float fao = mass_flux(uo[r], ro[r], P.r0, P.linear_mass);
            const float* cm = P.cM[F.side];
            const float* cr = P.cA[F.side];
            S.g[F.a][F.side][F.fi] = make_float2(fmo * cm[0] + fm_s * cm[1] + fao * cm[2] + fa_s * cm[3],
                                                 fmo * cr[0] + fm_s * cr[1] + fao * cr[2] + fa_s * cr[3] +
                                                     (F.side ? -0.5f : 0.5f) * (qo[r] + S.q[F.a][F.nf]));
        }
        __syncthreads();
        {
            // Line owners (see incr_stage_kernel); the per-axis results, already
            // times 1/w_a, reuse S.m (density) and S.q (momentum).  K = 5: one
            // warp per axis of each element slot, a lane per line; K = 6: the
            // element's 108 lines over its first 4 warps; K <= 4: the CTA's
            // threads over (slot, axis, line).
            constexpr int WPA = (K2 + 31) / 32;
            int a, t, ls;
            if constexpr (K >= 6) {
                // 3 K^2 = 108 tasks packed densely into 4 warps (an axis per
                // lane; the rows do not depend on the axis) instead of two
                // warps per axis with 28 idle lanes each
                a = n / K2;
                t = n % K2;
                ls = slot;
            } else if constexpr (K == 5) {
                const int w = n / 32;
                a = w / WPA;
                t = (w % WPA) * 32 + n % 32;
                ls = slot;
            } else {
                ls = threadIdx.x / (3 * K2);
                a = (threadIdx.x / K2) % 3;
                t = threadIdx.x % K2;
            }
            PlainSmem<float, K>& S = SM[ls < EPB ? ls : 0];
            if (ls < EPB && c0 + ls < T.e0 + T.count && a < 3 && t < K2) {
                const int st = axis_stride<K>(a);
                const int b0 = a == 0 ? t : (a == 1 ? (t % K) * K2 + (t / K) : t * K);
                float2 v[K];
#pragma unroll
                for (int j = 0; j < K; j++) v[j] = S.f[a][b0 + j * st];
                const float2 g0 = S.g[a][0][t], gN = S.g[a][1][t];
                const float iw = P.invw[a];
#pragma unroll
                for (int i = 0; i < K; i++) {
                    const float* row = ops.rows[i];  // constant-bank operands
                    float sm = row[K] * g0.x, sr = row[K] * g0.y;
                    sm += row[K + 1] * gN.x;
                    sr += row[K + 1] * gN.y;
#pragma unroll
                    for (int j = 0; j < K; j++) {
                        sm += row[j] * v[j].x;
                        sr += row[j] * v[j].y;
                    }
                    S.m[a][b0 + i * st] = iw * sr;
                    S.q[a][b0 + i * st] = iw * sm;
                }
            }
            __syncthreads();
        }
        if (act) {
            float r_rho = 0.f, r_u[3];
#pragma unroll
            for (int a = 0; a < 3; a++) {
                r_rho += S.m[a][n];
                r_u[a] = S.q[a][n];
            }
            const float ks = ca * sig;
            const float cbe = cb - ks, ce = eps - ks;
            const float r[4] = {r_rho, r_u[0], r_u[1], r_u[2]};
#pragma unroll
            for (int f = 0; f < 4; f++) {
                const size_t o = (size_t)f * P.fs + off;
                float d = ca * r[f] + ubv[f] * ce;
                if (inc) d += dv[f] * cbe;
                if (final_stage) {
                    const float y = d - cmp[f];
                    const float t = ubv[f] + y;
                    P.comp[o] = (t - ubv[f]) - y;
                    dout[o] = t;
                } else {
                    dout[o] = d;
                }
            }
        }
        // no barrier before the next pass: a thread reads only its own node's
        // S.m / S.q entries here, and the next pass rewrites them (by the same
        // thread) before its first barrier and the other entries only after it
    }
}

// Shared memory of one CTA of order K in phase PHASE.
template <int K, int PHASE>
__host__ __device__ constexpr size_t batch_smem_bytes()
{
    return bepb_of(K) * (PHASE == 0 ? sizeof(BatchGradSmem<K>) : sizeof(PlainSmem<float, K>));
}

// Resident CTAs per SM asked of the compiler for the gradient phase (register
// budget 65536 / (256 x 8) = 32; spills of 8-36 bytes at some orders): 136.3 G
// on config 4, against 131.1 G at 6 (42 registers) and 123.3 G with both
// phases in one kernel at the stage phase's budget.
constexpr int BATCH_GRAD_BLOCKS = 8;

// Resident CTAs per SM asked of the compiler for order K's stage phase (register
// 65536 / (threads x blocks)), chosen by measurement on config 4: 5 (48
// registers) for K = 2, 4 (no spills), 4 (64 registers) for K = 3, 5, which
// spill heavily at 48, and 5 CTAs of 224 threads (56 registers, no spills)
// for K = 6: 123.3 G, against 121.9 G with 6 CTAs at 48 registers and
// 121.5 G with 256-thread CTAs (with both phases in one kernel); with the
// phases apart, the K = 6 update at 48 registers (6 CTAs, 4 bytes of spills)
// measured 134.8 against 135.2 G.
__host__ __device__ constexpr int batch_min_blocks(int K, int phase)
{
    return phase == 0 ? BATCH_GRAD_BLOCKS : (K == 2 || K == 4 || K == 6 ? 5 : 4);
}

__device__ __forceinline__ void load_problem(BatchProblem& dst, const BatchProblem* src)
{
    const int* s = reinterpret_cast<const int*>(src);
    int* d = reinterpret_cast<int*>(&dst);
    for (int i = threadIdx.x; i < (int)(sizeof(BatchProblem) / sizeof(int)); i += blockDim.x) d[i] = s[i];
}

// One phase of one RK stage of every active problem of a group of order K:
// PHASE 0 the LDG gradient of every tile, PHASE 1 the stage update of every
// tile.  The two phases are separate launches (the kernel boundary is the
// barrier between them), so that groups can run as parallel branches of the
// step without any kernel waiting on another's blocks, and separate kernels,
// so that each gets its own register budget.  A persistent grid pulls the
// group's tiles from an atomic counter.
template <int K, int PHASE>
__global__ void __launch_bounds__(bthreads_of(K), batch_min_blocks(K, PHASE))
    batch_stage_kernel(BatchArgs A, const BatchOps ops)
{
    __shared__ __align__(16) unsigned char smraw[batch_smem_bytes<K, PHASE>()];
    __shared__ BatchProblem P;
    __shared__ int tile_idx;
    for (;;) {
        if (threadIdx.x == 0) tile_idx = atomicAdd(A.counters + PHASE, 1);
        __syncthreads();
        const int ti = tile_idx;
        if (ti >= A.n_tiles) break;
        const BatchTile T = A.tiles[A.tile0 + ti];
        load_problem(P, A.probs + T.prob);
        __syncthreads();
        if (P.active) {
            if constexpr (PHASE == 0) batch_grad_tile<K>(P, ops, T, A.stage, smraw);
            else batch_stage_tile<K>(P, ops, T, A.stage, smraw);
        }
        __syncthreads();
    }
}

// Writes one problem descriptor into its slot.  The descriptor travels as a
// kernel argument (copied at launch), so the host needs no page-locked
// staging and no synchronisation to add or retire a problem.
__global__ void batch_set_problem(BatchProblem* __restrict__ dst, const BatchProblem P)
{
    const int* s = reinterpret_cast<const int*>(&P);
    int* d = reinterpret_cast<int*>(dst);
    for (int i = threadIdx.x; i < (int)(sizeof(BatchProblem) / sizeof(int)); i += blockDim.x) d[i] = s[i];
}

// Per-problem bookkeeping around a step (one thread per problem).
__global__ void batch_step_begin(BatchProblem* probs, int n)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    BatchProblem& P = probs[i];
    if (!P.active) return;
    const double ts[3] = {P.t, P.t + P.dt, P.t + 0.5 * P.dt};
    for (int s = 0; s < 3; s++) {
        double p = 0.0;
        if (P.src_face >= 0 && ts[s] >= 0.0 && ts[s] <= P.src_T) {
            const double w = sin(3.14159265358979323846 * ts[s] / P.src_T);
            p = P.src_amp * w * w * sin(2.0 * 3.14159265358979323846 * P.src_freq * ts[s] + P.src_phase);
        }
        P.src_p[s] = (float)p;
    }
}

__global__ void batch_step_end(BatchProblem* probs, int n)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    BatchProblem& P = probs[i];
    if (!P.active) return;
    P.t += P.dt;
    P.cur ^= 1;
    P.steps_done++;
    if (--P.steps_left <= 0) P.active = 0;
}

}  // namespace dg
