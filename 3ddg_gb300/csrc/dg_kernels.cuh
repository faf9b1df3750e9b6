// sm_103a kernels for one stage of the DG right-hand side and its RK update.
//
// Two launches per RK stage (one without diffusion):
//   ldg_gradient_kernel  Q_a = d(drho)/dx_a by LDG with the central flux
//                        (Element::OperateQFromDRho, cppsrc/Element.cpp:623-690)
//   stage_kernel         volume + face terms of the advection operator
//                        (Element::OperateUFromV, cppsrc/Element.cpp:475-620),
//                        LDG divergence (Element::OperateDRhoFromQ, :691-758),
//                        sponge (Element::OperateSponge, :760-781) and the RK
//                        stage combination (Element::selfWeightedAdd, :288-307)
//                        fused into one pass over the state.
//
// Mapping: one thread per node, one warp-aligned slice of NPT threads per
// element, EPB elements per CTA.  Each element stages its volume fluxes and
// its face fluxes in shared memory; the line sums along each axis read shared
// memory with D = M^-1 S held in registers.  The reference's per-line QR solve
// of (M q w) x = S q f - F becomes x = (1/w) D f - (1/(q w)) (M^-1 e_0 F_0 +
// M^-1 e_N F_N): D and the lift columns are computed once on the host in FP64.
// Neighbour face values are read straight from the neighbour element (same
// block or another block of the same HBM pool) through the face table, which
// replaces the halo ring and Grid::communicate.
#pragma once

#include <cstddef>
#include <cstdint>

namespace dg {

__host__ __device__ constexpr int npt_of(int K) { return (K * K * K + 31) / 32 * 32; }
__host__ __device__ constexpr int epb_of(int K) { return K <= 3 ? 4 : (K == 4 ? 2 : 1); }

// Per-problem operator constants, passed by value (kernel parameter space).
template <typename T, int K>
struct OpConst {
    T D[K][K];             // D = M^-1 S on the unit interval
    T L0[K], LN[K];        // lift columns M^-1 e_0, M^-1 e_N
    T inv_w[3];            // 1 / w_a
    T s_mom[3];            // -1 / (rho0 w_a): lift scale of the momentum equation
    T s_mass[3];           // -rho0 / w_a:     lift scale of the mass equation
    T s_diff[3];           // -D / w_a:        scale of the LDG divergence
    T cL0[4], cL1[4];      // left-face flux coefficients, modes 0 and 1
    T cR0[4], cR1[4];      // right-face flux coefficients, modes 0 and 1
    T ba, inv_r0, c2_r0, r0;  // momentum / mass flux constants
    T inv_c2, inv_z;       // source exterior state: drho = p / c^2, u = p / (rho0 c)
    int linear_mass;       // B/A == 0 selects u*rho0 (cppsrc/kernelFuncs.cpp:25)
    int dense_lift;        // 0 when M is diagonal (lift touches end nodes only)
};

// Mesh arrays on the device (see mesh.h).
template <typename T>
struct MeshDev {
    const int* nbr;        // n_elem * 6, faces -X +X -Y +Y -Z +Z
    const T* sigma;        // n_elem
    const T* bnd_ic;       // n_bnd * 2 * K^2
    const T* bnd_ap;       // n_bnd * K^2
    const int* bnd_src;    // n_bnd: 1 on the source face
    int n_elem;
    int ic_live;           // exterior = IC halo values (first stage after creation)
    T src_p;               // source pressure at this stage's time
};

// Stage input/output.  PLAIN (FP64 method): the stage input is ``src``,
//   dst = ca * R + cb * src (+ cc * old).
// INCR (FP32 form): the stage input is u + d (d = ``inc``, absent in stage 1),
//   d_out = ca * R + cb * d + eps * u; the final stage adds d_out to u with a
//   Kahan-compensated sum into ``dst`` (the other u buffer) and ``comp``.
template <typename T>
struct StageIO {
    const T* src;
    const T* inc;
    const T* old;
    T* dst;
    T* comp;
    const T* q;            // LDG gradient, 3 fields
    T* q_out;              // gradient kernel output
    size_t fs;             // field stride (n_elem * NP)
    int np;                // nodes per element in memory
    T ca, cb, cc, eps;
    int final_stage;
};

template <typename T>
__device__ __forceinline__ T momentum_flux(T d, const T ba, const T inv_r0, const T c2_r0)
{
    // cppsrc/kernelFuncs.cpp:19-20: (d + d*d*B/A*0.5*(1/rho0)) * (c*c/rho0)
    T t = d * d;
    t = t * ba;
    t = t * T(0.5);
    t = t * inv_r0;
    return (d + t) * c2_r0;
}

template <typename T>
__device__ __forceinline__ T mass_flux(T u, T d, const T r0, int linear)
{
    // cppsrc/kernelFuncs.cpp:23-29
    return linear ? u * r0 : u * (d + r0);
}

template <typename T, int K>
struct StageSmem {
    T fm[npt_of(K)];
    T fa[3][npt_of(K)];
    T qa[3][npt_of(K)];
    T fl[3][2][3][K * K];  // [axis][side][mom, mass, diff][face node]
};

template <typename T, int K>
struct GradSmem {
    T r[npt_of(K)];
    T fl[3][2][K * K];
};

template <bool INCR, typename T>
__device__ __forceinline__ T load_in(const StageIO<T>& io, int f, size_t off)
{
    T v = __ldg(io.src + (size_t)f * io.fs + off);
    if (INCR && io.inc) v += __ldg(io.inc + (size_t)f * io.fs + off);
    return v;
}

// Exterior value at a domain-boundary face node: the tone burst on the source
// face, else the IC halo values during the first stage, else zero.
template <typename T, int K>
__device__ __forceinline__ void exterior(const MeshDev<T>& m, const OpConst<T, K>& C, int slot,
                                         int side, int fi, T& ro, T& uo)
{
    if (m.bnd_src[slot]) {
        T p = m.src_p * m.bnd_ap[(size_t)slot * K * K + fi];
        ro = p * C.inv_c2;
        uo = (side == 0 ? p : -p) * C.inv_z;
    } else if (m.ic_live) {
        ro = m.bnd_ic[((size_t)slot * 2 + 0) * K * K + fi];
        uo = m.bnd_ic[((size_t)slot * 2 + 1) * K * K + fi];
    } else {
        ro = T(0);
        uo = T(0);
    }
}

template <int K>
__device__ __forceinline__ int axis_stride(int a)
{
    return a == 0 ? K * K : (a == 1 ? K : 1);
}

// ---------------------------------------------------------------------------
// LDG gradient: Q_a = -(1/w_a) (D drho + M^-1 e_0 F_0 + M^-1 e_N F_N) with the
// central flux F_0 = (drho_o[N] + drho_s[0]) / 2, F_N = -(drho_s[N] + drho_o[0]) / 2.
// ---------------------------------------------------------------------------
template <typename T, int K, bool INCR>
__global__ void __launch_bounds__(npt_of(K) * epb_of(K))
ldg_gradient_kernel(StageIO<T> io, MeshDev<T> m, OpConst<T, K> C)
{
    constexpr int K2 = K * K, K3 = K * K * K;
    __shared__ GradSmem<T, K> sm_all[epb_of(K)];
    GradSmem<T, K>& S = sm_all[threadIdx.y];
    const int n = threadIdx.x;
    const int e = blockIdx.x * epb_of(K) + threadIdx.y;
    const bool act = n < K3 && e < m.n_elem;
    const int c[3] = {n / K2, (n / K) % K, n % K};
    T rho = T(0);
    if (act) rho = load_in<INCR>(io, 0, (size_t)e * io.np + n);
    S.r[n] = rho;
    if (act) {
#pragma unroll
        for (int a = 0; a < 3; a++) {
            if (c[a] != 0 && c[a] != K - 1) continue;
            const int side = c[a] == 0 ? 0 : 1;
            const int fi = c[(a + 1) % 3] * K + c[(a + 2) % 3];
            const int code = __ldg(m.nbr + (size_t)e * 6 + 2 * a + side);
            T ro, uo;
            if (code >= 0) {
                const int nn = n + ((side ? 0 : K - 1) - c[a]) * axis_stride<K>(a);
                ro = load_in<INCR>(io, 0, (size_t)code * io.np + nn);
            } else {
                exterior<T, K>(m, C, -1 - code, side, fi, ro, uo);
            }
            S.fl[a][side][fi] = side == 0 ? T(0.5) * (ro + rho) : T(-0.5) * (rho + ro);
        }
    }
    __syncthreads();
    if (!act) return;
#pragma unroll
    for (int a = 0; a < 3; a++) {
        const int st = axis_stride<K>(a);
        const int ia = c[a];
        const int base = n - ia * st;
        const int fi = c[(a + 1) % 3] * K + c[(a + 2) % 3];
        T s = T(0);
#pragma unroll
        for (int j = 0; j < K; j++) s += C.D[ia][j] * S.r[base + j * st];
        T lf;
        if (C.dense_lift) lf = C.L0[ia] * S.fl[a][0][fi] + C.LN[ia] * S.fl[a][1][fi];
        else lf = (ia == 0 ? C.L0[ia] * S.fl[a][0][fi] : T(0)) + (ia == K - 1 ? C.LN[ia] * S.fl[a][1][fi] : T(0));
        io.q_out[(size_t)a * io.fs + (size_t)e * io.np + n] = T(-1) * (C.inv_w[a] * (s + lf));
    }
}

// ---------------------------------------------------------------------------
// One RK stage: R = L(stage input), then the stage combination.
// ---------------------------------------------------------------------------
template <typename T, int K, bool DIFF, bool INCR>
__global__ void __launch_bounds__(npt_of(K) * epb_of(K))
stage_kernel(StageIO<T> io, MeshDev<T> m, OpConst<T, K> C, int do_adv, int do_sponge)
{
    constexpr int K2 = K * K, K3 = K * K * K;
    __shared__ StageSmem<T, K> sm_all[epb_of(K)];
    StageSmem<T, K>& S = sm_all[threadIdx.y];
    const int n = threadIdx.x;
    const int e = blockIdx.x * epb_of(K) + threadIdx.y;
    const bool act = n < K3 && e < m.n_elem;
    const int c[3] = {n / K2, (n / K) % K, n % K};
    const size_t off = (size_t)e * io.np + n;

    T rho = T(0), u[3] = {T(0), T(0), T(0)}, q[3] = {T(0), T(0), T(0)};
    if (act) {
        rho = load_in<INCR>(io, 0, off);
#pragma unroll
        for (int a = 0; a < 3; a++) u[a] = load_in<INCR>(io, 1 + a, off);
        if (DIFF)
#pragma unroll
            for (int a = 0; a < 3; a++) q[a] = __ldg(io.q + (size_t)a * io.fs + off);
    }
    const T fmom = momentum_flux(rho, C.ba, C.inv_r0, C.c2_r0);
    T fmass[3];
#pragma unroll
    for (int a = 0; a < 3; a++) fmass[a] = mass_flux(u[a], rho, C.r0, C.linear_mass);
    S.fm[n] = fmom;
#pragma unroll
    for (int a = 0; a < 3; a++) {
        S.fa[a][n] = fmass[a];
        if (DIFF) S.qa[a][n] = q[a];
    }

    // Face fluxes: the thread owning a face node evaluates that face's numerical
    // flux for its line (impedance upwind for advection, central for LDG).
    if (act) {
#pragma unroll
        for (int a = 0; a < 3; a++) {
            if (c[a] != 0 && c[a] != K - 1) continue;
            const int side = c[a] == 0 ? 0 : 1;
            const int fi = c[(a + 1) % 3] * K + c[(a + 2) % 3];
            const int code = __ldg(m.nbr + (size_t)e * 6 + 2 * a + side);
            T ro, uo, qo = T(0);
            if (code >= 0) {
                const int nn = n + ((side ? 0 : K - 1) - c[a]) * axis_stride<K>(a);
                const size_t o2 = (size_t)code * io.np + nn;
                ro = load_in<INCR>(io, 0, o2);
                uo = load_in<INCR>(io, 1 + a, o2);
                if (DIFF) qo = __ldg(io.q + (size_t)a * io.fs + o2);
            } else {
                exterior<T, K>(m, C, -1 - code, side, fi, ro, uo);
            }
            const T fmo = momentum_flux(ro, C.ba, C.inv_r0, C.c2_r0);
            const T fao = mass_flux(uo, ro, C.r0, C.linear_mass);
            if (side == 0) {
                S.fl[a][0][0][fi] = T(-1) * (fmo * C.cL0[0] + fmom * C.cL0[1] + fao * C.cL0[2] + fmass[a] * C.cL0[3]);
                S.fl[a][0][1][fi] = T(-1) * (fao * C.cL1[0] + fmass[a] * C.cL1[1] + fmo * C.cL1[2] + fmom * C.cL1[3]);
                if (DIFF) S.fl[a][0][2][fi] = T(0.5) * (qo + q[a]);
            } else {
                S.fl[a][1][0][fi] = fmom * C.cR0[0] + fmo * C.cR0[1] + fmass[a] * C.cR0[2] + fao * C.cR0[3];
                S.fl[a][1][1][fi] = fmass[a] * C.cR1[0] + fao * C.cR1[1] + fmom * C.cR1[2] + fmo * C.cR1[3];
                if (DIFF) S.fl[a][1][2][fi] = T(-0.5) * (q[a] + qo);
            }
        }
    }
    __syncthreads();
    if (!act) return;

    T r_rho = T(0), r_u[3] = {T(0), T(0), T(0)};
    // LDG divergence first, as the reference accumulates it (cppsrc/Grid.cpp:674-689).
    if (DIFF) {
#pragma unroll
        for (int a = 0; a < 3; a++) {
            const int st = axis_stride<K>(a), ia = c[a], base = n - ia * st;
            const int fi = c[(a + 1) % 3] * K + c[(a + 2) % 3];
            T s = T(0);
#pragma unroll
            for (int j = 0; j < K; j++) s += C.D[ia][j] * S.qa[a][base + j * st];
            T lf;
            if (C.dense_lift) lf = C.L0[ia] * S.fl[a][0][2][fi] + C.LN[ia] * S.fl[a][1][2][fi];
            else lf = (ia == 0 ? C.L0[ia] * S.fl[a][0][2][fi] : T(0)) + (ia == K - 1 ? C.LN[ia] * S.fl[a][1][2][fi] : T(0));
            r_rho += C.s_diff[a] * (s + lf);
        }
    }
    if (do_adv) {
#pragma unroll
        for (int a = 0; a < 3; a++) {
            const int st = axis_stride<K>(a), ia = c[a], base = n - ia * st;
            const int fi = c[(a + 1) % 3] * K + c[(a + 2) % 3];
            T sm = T(0), sa = T(0);
#pragma unroll
            for (int j = 0; j < K; j++) {
                sm += C.D[ia][j] * S.fm[base + j * st];
                sa += C.D[ia][j] * S.fa[a][base + j * st];
            }
            T lm, la;
            if (C.dense_lift) {
                lm = C.L0[ia] * S.fl[a][0][0][fi] + C.LN[ia] * S.fl[a][1][0][fi];
                la = C.L0[ia] * S.fl[a][0][1][fi] + C.LN[ia] * S.fl[a][1][1][fi];
            } else {
                lm = (ia == 0 ? C.L0[ia] * S.fl[a][0][0][fi] : T(0)) + (ia == K - 1 ? C.LN[ia] * S.fl[a][1][0][fi] : T(0));
                la = (ia == 0 ? C.L0[ia] * S.fl[a][0][1][fi] : T(0)) + (ia == K - 1 ? C.LN[ia] * S.fl[a][1][1][fi] : T(0));
            }
            r_u[a] += C.inv_w[a] * sm + C.s_mom[a] * lm;
            r_rho += C.inv_w[a] * sa + C.s_mass[a] * la;
        }
    }
    if (do_sponge) {
        const T sg = __ldg(m.sigma + e);
#pragma unroll
        for (int a = 0; a < 3; a++) r_u[a] += T(-1) * u[a] * sg;
        r_rho += T(-1) * rho * sg;
    }

    const T r[4] = {r_rho, r_u[0], r_u[1], r_u[2]};
    if (!INCR) {
        const T s4[4] = {rho, u[0], u[1], u[2]};
#pragma unroll
        for (int f = 0; f < 4; f++) {
            const size_t o = (size_t)f * io.fs + off;
            T v = r[f] * io.ca + s4[f] * io.cb;
            if (io.old) v = v + io.old[o] * io.cc;
            io.dst[o] = v;
        }
    } else {
#pragma unroll
        for (int f = 0; f < 4; f++) {
            const size_t o = (size_t)f * io.fs + off;
            const T ub = __ldg(io.src + o);
            T d = r[f] * io.ca;
            if (io.inc) d += io.cb * __ldg(io.inc + o);
            if (io.final_stage) {
                d += io.eps * ub;
                // Kahan-compensated u <- u + d
                const T y = d - io.comp[o];
                const T t = ub + y;
                io.comp[o] = (t - ub) - y;
                io.dst[o] = t;
            } else {
                io.dst[o] = d;
            }
        }
    }
}

// Element-major state  <->  node-duplicated [X][Y][Z] grid layout (the
// reference's HDF5 dataset order, cppsrc/HDF5Functions.cpp:173-208).
struct GridMap {
    int K, nb[3], ne[3], E[3], elem_per_block;
};

__device__ __forceinline__ size_t grid_index(const GridMap& g, int e, int n)
{
    const int blk = e / g.elem_per_block, le = e % g.elem_per_block;
    const int b0 = blk / (g.nb[1] * g.nb[2]), b1 = (blk / g.nb[2]) % g.nb[1], b2 = blk % g.nb[2];
    const int l0 = le / (g.ne[1] * g.ne[2]), l1 = (le / g.ne[2]) % g.ne[1], l2 = le % g.ne[2];
    const int K = g.K;
    const size_t ii = (size_t)(b0 * g.ne[0] + l0) * K + n / (K * K);
    const size_t jj = (size_t)(b1 * g.ne[1] + l1) * K + (n / K) % K;
    const size_t kk = (size_t)(b2 * g.ne[2] + l2) * K + n % K;
    return (ii * ((size_t)g.E[1] * K) + jj) * ((size_t)g.E[2] * K) + kk;
}

template <typename T>
__global__ void pack_grid_kernel(const T* __restrict__ state, size_t fs, int np, int nfields,
                                 GridMap g, int n_elem, double* __restrict__ out, size_t gsize)
{
    const int K3 = g.K * g.K * g.K;
    const long long total = (long long)n_elem * K3;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const int e = (int)(i / K3), n = (int)(i % K3);
        const size_t gi = grid_index(g, e, n);
        for (int f = 0; f < nfields; f++)
            out[(size_t)f * gsize + gi] = (double)state[(size_t)f * fs + (size_t)e * np + n];
    }
}

template <typename T>
__global__ void unpack_grid_kernel(T* __restrict__ state, size_t fs, int np, int nfields,
                                   GridMap g, int n_elem, const double* __restrict__ in, size_t gsize)
{
    const int K3 = g.K * g.K * g.K;
    const long long total = (long long)n_elem * K3;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const int e = (int)(i / K3), n = (int)(i % K3);
        const size_t gi = grid_index(g, e, n);
        for (int f = 0; f < nfields; f++)
            state[(size_t)f * fs + (size_t)e * np + n] = (T)in[(size_t)f * gsize + gi];
    }
}

}  // namespace dg
