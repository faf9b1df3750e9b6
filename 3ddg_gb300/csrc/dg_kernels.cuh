// sm_103a kernels for one stage of the DG right-hand side and its RK update.
//
// Two launches per RK stage (one without diffusion):
//   ldg_gradient_kernel  G_a = -D_c d(drho)/dx_a by LDG with the central flux
//                        (Element::OperateQFromDRho, cppsrc/Element.cpp:623-690;
//                        stored pre-multiplied by -D_c, the diffusive flux)
//   stage_kernel (FP64), incr_stage_kernel (FP32 increment form)
//                        volume + face terms of the advection operator
//                        (Element::OperateUFromV, cppsrc/Element.cpp:475-620),
//                        LDG divergence (Element::OperateDRhoFromQ, :691-758),
//                        sponge (Element::OperateSponge, :760-781) and the RK
//                        stage combination (Element::selfWeightedAdd, :288-307)
//                        fused into one pass over the state.
//
// Mapping: one thread per node, one warp-aligned slice of NPT threads per
// element, EPB elements per CTA.  Each thread loads its node (and the
// neighbour values its face work needs) before the first use; the element
// stages its volume fluxes in shared memory; face fluxes and line sums follow
// after barriers.  The reference's per-line QR solve of
// (M q w) x = S q f - F becomes
//     x = (1/w) D f - (1/(q w)) (M^-1 e_0 F_0 + M^-1 e_N F_N),  D = M^-1 S,
// with D and the lift columns computed once on the host in FP64.
//
// FP64 (bound by the FP64 pipe): every constant factor is folded on the host
// into the per-launch operator (OpConst): the RK stage weight ca, 1/w_a and
// the equations' lift scales go into per-axis copies of D and into the
// face-flux coefficients, the gradient carries -D_c so that the LDG
// divergence and the mass-flux divergence share one line sum, and the sponge
// folds into the RK combination (its per-element weight tabulated by the
// host).  The element's face nodes are dealt out densely to its threads so
// that no warp issues face arithmetic for lanes that have none; each stage
// writes the volume fluxes of its output for the next stage to read (flux
// modes), so no face neighbour's flux is evaluated twice; and at K = 5 the
// line sums use the even-odd split of the centro-antisymmetric D (LineEO),
// with line owners packed densely two elements per CTA, instead of per-node
// sums of 2 (K + 2) FMAs per axis.
//
// FP32 (bound by the L1 data pipe, load latency and issue): for K >= 5 line
// owners (a warp per axis, a lane per line) evaluate their line's two face
// terms and its K outputs with the operator as kernel parameters, instead of
// every node summing its own three lines from shared memory.
//
// Neighbour face values are read straight from the neighbour element (same
// block or another block of the same HBM pool) through the face table, which
// replaces the halo ring and Grid::communicate.
#pragma once

#include <cmath>
#include <cstddef>
#include <cstdint>

namespace dg {

__host__ __device__ constexpr int npt_of(int K) { return (K * K * K + 31) / 32 * 32; }
__host__ __device__ constexpr int epb_of(int K) { return K <= 3 ? 4 : (K == 4 ? 2 : 1); }

// A 16-byte vector of T (the widest per-thread global load).
template <typename T>
struct Vec16;
template <>
struct Vec16<float> {
    using type = float4;
};
template <>
struct Vec16<double> {
    using type = double2;
};

// Length of one operator row: K entries of D, the two lift entries, padded to
// whole 16-byte vectors.
template <typename T, int K>
__host__ __device__ constexpr int oprow_len()
{
    return (K + 2 + (int)(16 / sizeof(T)) - 1) / (int)(16 / sizeof(T)) * (int)(16 / sizeof(T));
}

// Per-launch operator constants, in device memory.
//   stage kernel:    D[a] = ca D / w_a;   cM, cA: face coefficients of the
//                    momentum / mass equations times ca * (lift scale);
//                    cQ[a] = (+0.5, -0.5) ca / w_a (central flux of G).
//   gradient kernel: D[a] = D_c D / w_a;  lift columns times the central-flux
//                    factors (+0.5, -0.5) D_c / w_a (cQ unused).
// rows[a][i] = (D[a][i][0..K-1], L0[i], LN[i], 0...) with the lift columns
// L0 = M^-1 e_0, LN = M^-1 e_N, so that a thread loads its row of each axis
// with one or two 16-byte loads.
// Face coefficients act on (f_mom other, f_mom self, f_mass other, f_mass self).
template <typename T, int K>
struct OpConst {
    alignas(16) T rows[3][K][oprow_len<T, K>()];
    T cM[3][2][4];
    T cA[3][2][4];
    T cQ[3][2];
    T k1, k2;              // f_mom(rho) = rho (k1 + k2 rho) = c^2/rho0 (rho + B/A rho^2 / (2 rho0))
    T r0;                  // f_mass(u, rho) = u (rho + rho0), or u rho0 when B/A = 0
    T inv_c2, inv_z;       // source exterior state: drho = p / c^2, u = p / (rho0 c)
    int linear_mass;
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

// Stage input/output.  R' = ca R_ops is what the folded operator produces
// (R_ops: advection + diffusion, without the sponge).
//   PLAIN (FP64 method), stage input s = ``src``:
//       dst = R' + s (cb - ca sigma) + cc old         (= ca R + cb s + cc old)
//   INCR (FP32 form), stage input s = u + d (u = ``src``, d = ``inc``, absent
//   in stage 1):
//       d_out = R' + d (cb - ca sigma) + u (eps - ca sigma)
//                                                     (= ca R + cb d + eps u)
//       and in the final stage u <- u + d_out with a Kahan-compensated sum
//       into ``dst`` (the other u buffer) and ``comp``.
template <typename T>
struct StageIO {
    const T* src;
    const T* inc;
    const T* old;
    T* dst;
    T* comp;
    const T* q;            // LDG gradient (times -D_c), 3 fields
    T* q_out;              // gradient kernel output
    const T* elem_b;       // PLAIN: cb - ca sigma per element for this stage (null: from sigma)
    const T* flux_in;      // PLAIN, flux mode 2: volume fluxes of src (f_mom, f_mass x, y, z)
    T* flux_out;           // PLAIN, flux modes 1, 2: the same of dst
    size_t fs;             // field stride (n_elem * NP)
    int np;                // nodes per element in memory
    T ca, cb, cc, eps;
    int final_stage;
    // PLAIN, PACK: the output also written in host order ([X][Y][Z] per
    // field, fields gsize apart) for a download
    double* pack;
    GridMap pack_map;
    size_t pack_gsize;
};

template <typename T>
__device__ __forceinline__ T momentum_flux(T d, const T k1, const T k2)
{
    return d * (k1 + k2 * d);
}

template <typename T>
__device__ __forceinline__ T mass_flux(T u, T d, const T r0, int linear)
{
    // cppsrc/kernelFuncs.cpp:23-29
    return linear ? u * r0 : u * (d + r0);
}

template <typename T>
struct Pair;
template <>
struct Pair<float> {
    using type = float2;
};
template <>
struct Pair<double> {
    using type = double2;
};

// Volume-flux output of the FP64 unpack kernels (f null: none): the fluxes
// of the state they write, so that the first stage after an upload reads
// them like any later stage.
template <typename T>
struct FluxOut {
    T* f;
    T k1, k2, r0;
    int linear;
};

// The flux constants of the stage operators and of FluxOut, from one place
// so that both evaluate bit-identical fluxes.
template <typename T>
inline FluxOut<T> flux_consts(T* f, double rho0, double c0, double b_over_a)
{
    FluxOut<T> o;
    o.f = f;
    o.k1 = (T)(c0 * c0 / rho0);
    o.k2 = (T)(b_over_a * 0.5 * c0 * c0 / (rho0 * rho0));
    o.r0 = (T)rho0;
    o.linear = b_over_a == 0.0 ? 1 : 0;
    return o;
}

template <typename T>
__device__ __forceinline__ void write_fluxes(const FluxOut<T>& fo, size_t fs, size_t o, T d, const T u[3])
{
    fo.f[o] = momentum_flux(d, fo.k1, fo.k2);
#pragma unroll
    for (int a = 0; a < 3; a++) fo.f[(size_t)(1 + a) * fs + o] = mass_flux(u[a], d, fo.r0, fo.linear);
}

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
__host__ __device__ constexpr int axis_stride(int a)
{
    return a == 0 ? K * K : (a == 1 ? K : 1);
}

// Face nodes of an element, numbered t = (2 a + side) K^2 + fi for the faces
// -X +X -Y +Y -Z +Z, fi = c[(a+1)%3] K + c[(a+2)%3]: the element's node on
// the face (nf) and the neighbour's node across it (nn, in the neighbour).
// The decoding is tabulated per order at compile time (one packed word per
// face node: a 2 bits, side 1, fi 7, nf 10, nn 10), so that a thread loads its
// face nodes' entries (coalesced) instead of redoing the integer arithmetic.
template <int K>
struct FaceTable {
    int v[6 * K * K];
    constexpr FaceTable() : v{}
    {
        constexpr int K2 = K * K;
        for (int t = 0; t < 6 * K2; t++) {
            const int a = t / (2 * K2), side = (t / K2) & 1, fi = t % K2, p = side ? K - 1 : 0;
            const int nf = a == 0 ? p * K2 + fi : (a == 1 ? (fi % K) * K2 + p * K + fi / K : fi * K + p);
            const int nn = nf + (side ? -(K - 1) : (K - 1)) * (a == 0 ? K2 : (a == 1 ? K : 1));
            v[t] = a | (side << 2) | (fi << 3) | (nf << 10) | (nn << 20);
        }
    }
};
template <int K>
__device__ const FaceTable<K> kFaceTable{};

// The same decoding by integer arithmetic (no memory access).
template <int K>
struct FaceNodeArith {
    int a, side, fi, nf, nn;
    __device__ __forceinline__ explicit FaceNodeArith(int t)
    {
        constexpr int K2 = K * K;
        a = t / (2 * K2);
        side = (t / K2) & 1;
        fi = t % K2;
        const int p = side ? K - 1 : 0;
        nf = a == 0 ? p * K2 + fi : (a == 1 ? (fi % K) * K2 + p * K + fi / K : fi * K + p);
        nn = nf + (side ? -(K - 1) : (K - 1)) * axis_stride<K>(a);
    }
};

template <int K>
struct FaceNode {
    int a, side, fi, nf, nn;
    __device__ __forceinline__ explicit FaceNode(int t)
    {
        const int w = __ldg(&kFaceTable<K>.v[t]);
        a = w & 3;
        side = (w >> 2) & 1;
        fi = (w >> 3) & 127;
        nf = (w >> 10) & 1023;
        nn = (w >> 20) & 1023;
    }
};

// ---------------------------------------------------------------------------
// LDG gradient, stored as G_a = -D_c Q_a = (D_c / w_a)(D drho + M^-1 e_0 F_0 +
// M^-1 e_N F_N) with the central flux F_0 = (drho_o[N] + drho_s[0]) / 2,
// F_N = -(drho_s[N] + drho_o[0]) / 2.
// ---------------------------------------------------------------------------
// Each thread's rows of the per-launch operator (its index along each axis),
// loaded once through L1 into registers.  The operator lives in global memory:
// indexing kernel-parameter space with a per-thread index would serialise on
// the address-divergence unit.
template <typename T, int K>
struct OpRows {
    T d[3][K], l0[3], ln[3];
    __device__ __forceinline__ void load(const OpConst<T, K>& C, const int c[3], bool act)
    {
        using V = typename Vec16<T>::type;
        constexpr int RL = oprow_len<T, K>(), NV = RL * (int)sizeof(T) / 16;
#pragma unroll
        for (int a = 0; a < 3; a++) {
            const int ia = act ? c[a] : 0;
            T row[RL];
            const V* src = reinterpret_cast<const V*>(C.rows[a][ia]);
#pragma unroll
            for (int v = 0; v < NV; v++) reinterpret_cast<V*>(row)[v] = __ldg(src + v);
#pragma unroll
            for (int j = 0; j < K; j++) d[a][j] = row[j];
            l0[a] = row[K];
            ln[a] = row[K + 1];
        }
    }
};

// First node of line t along axis A (lines numbered like the face nodes fi),
// for the line owners below.
template <int A, int K>
__device__ __forceinline__ int line_base(int t)
{
    return A == 0 ? t : (A == 1 ? (t % K) * K * K + t / K : t * K);
}

// Even-odd form of one axis's line operator (FP64 line owners).  D is
// centro-antisymmetric, D[K-1-i][K-1-j] = -D[i][j], and the lift columns are
// mirrored, L0[K-1-i] = SIG LN[i]; with e_j = v_j + v_{K-1-j},
// o_j = v_j - v_{K-1-j} (j < H = K/2), s = f0 + fN, d = f0 - fN:
//   P_i = sum_j E[i][j] e_j + Dc[i] v_H,  Q_i = sum_j O[i][j] o_j,
//   out_i = P_i + Q_i,  out_{K-1-i} = Q_i - P_i   (i < H; the lift terms
//   A s, B d are added to P or Q by SIG),
//   out_H = sum_j Dm[j] o_j + Lm (s or d)   (K odd),
// E = (D[i][j] + D[i][K-1-j]) / 2, O = (D[i][j] - D[i][K-1-j]) / 2,
// A = (L0 + LN) / 2, B = (L0 - LN) / 2: at K = 5, 27 FP64 instructions per
// line and field instead of the 35 of K per-node sums with two lift terms.
template <int K>
struct LineEOAxis {
    static constexpr int H = K / 2;
    double E[H][H], O[H][H];
    double Dc[H];          // D[i][H], K odd
    double Al[H], Bl[H];   // lift combinations
    double Dm[H];          // D[H][j], K odd
    double Lm;             // L0[H], K odd
};
template <int K>
struct LineEO {
    LineEOAxis<K> ax[3];
};

// One line of one field.  The line owners of a warp cover more than one axis
// (3 K^2 tasks packed densely), so the axis is a runtime value and its
// coefficients X come from shared memory: every lane runs the same FP64
// instructions.
template <int K, int SIG>
__device__ __forceinline__ void eo_apply(const LineEOAxis<K>& X, const double v[K], double f0, double fN,
                                         double out[K])
{
    constexpr int H = K / 2;
    double e[H], o[H];
#pragma unroll
    for (int j = 0; j < H; j++) {
        e[j] = v[j] + v[K - 1 - j];
        o[j] = v[j] - v[K - 1 - j];
    }
    const double s = f0 + fN, d = f0 - fN;
#pragma unroll
    for (int i = 0; i < H; i++) {
        double P = X.E[i][0] * e[0], Q = X.O[i][0] * o[0];
#pragma unroll
        for (int j = 1; j < H; j++) {
            P += X.E[i][j] * e[j];
            Q += X.O[i][j] * o[j];
        }
        if (K & 1) P += X.Dc[i] * v[H];
        if (SIG > 0) {
            P += X.Bl[i] * d;
            Q += X.Al[i] * s;
        } else {
            P += X.Al[i] * s;
            Q += X.Bl[i] * d;
        }
        out[i] = P + Q;
        out[K - 1 - i] = Q - P;
    }
    if (K & 1) {
        double c = X.Lm * (SIG > 0 ? s : d);
#pragma unroll
        for (int j = 0; j < H; j++) c += X.Dm[j] * o[j];
        out[H] = c;
    }
}

// Line owner with its own face terms (FP32, K >= 5): the two ends of line t
// along axis A are the face nodes (A, 0, t) and (A, 1, t), so the owner
// evaluates both numerical fluxes itself (neighbour values ro/uo/qo[side],
// prefetched; own values from shared memory) and then the line sums.  The
// face coefficients come from kernel parameters with a compile-time axis.
template <int A, bool DIFF, typename T, int K, typename Smem>
__device__ __forceinline__ void stage_line_faces(const OpConst<T, K>& Cv, Smem& S, int t, const T ro[2],
                                                 const T uo[2], const T qo[2], int do_adv)
{
    constexpr int st = axis_stride<K>(A);
    const int b0 = line_base<A, K>(t);
    typename Pair<T>::type g[2];
#pragma unroll
    for (int side = 0; side < 2; side++) {
        const int nf = b0 + (side ? (K - 1) * st : 0);
        const T fm_s = S.f[A][nf].x, fa_s = S.m[A][nf];
        T gm = T(0), gr = T(0);
        if (do_adv) {
            const T fmo = momentum_flux(ro[side], Cv.k1, Cv.k2);
            const T fao = mass_flux(uo[side], ro[side], Cv.r0, Cv.linear_mass);
            const T* cm = Cv.cM[A][side];
            const T* cr = Cv.cA[A][side];
            gm = fmo * cm[0] + fm_s * cm[1] + fao * cm[2] + fa_s * cm[3];
            gr = fmo * cr[0] + fm_s * cr[1] + fao * cr[2] + fa_s * cr[3];
        }
        if (DIFF) gr += Cv.cQ[A][side] * (qo[side] + S.q[A][nf]);
        g[side].x = gm;
        g[side].y = gr;
    }
    typename Pair<T>::type v[K];
#pragma unroll
    for (int j = 0; j < K; j++) v[j] = S.f[A][b0 + j * st];
#pragma unroll
    for (int i = 0; i < K; i++) {
        const T* row = Cv.rows[A][i];
        T sm = row[K] * g[0].x, sr = row[K] * g[0].y;
        sm += row[K + 1] * g[1].x;
        sr += row[K + 1] * g[1].y;
#pragma unroll
        for (int j = 0; j < K; j++) {
            sm += row[j] * v[j].x;
            sr += row[j] * v[j].y;
        }
        S.m[A][b0 + i * st] = sr;
        S.q[A][b0 + i * st] = sm;
    }
}

// The same for the LDG gradient: central flux of drho at both ends; the
// owner stores its line's K values of G_A at q_elem (the element's G_A).
template <int A, typename T, int K, typename Smem>
__device__ __forceinline__ void grad_line_faces(const OpConst<T, K>& Cv, const Smem& S, int t, const T ro[2],
                                                T* __restrict__ q_elem)
{
    constexpr int st = axis_stride<K>(A);
    const int b0 = line_base<A, K>(t);
    T v[K];
#pragma unroll
    for (int j = 0; j < K; j++) v[j] = S.r[b0 + j * st];
    const T f0 = ro[0] + v[0], fN = ro[1] + v[K - 1];  // flux factors are in the lift columns
#pragma unroll
    for (int i = 0; i < K; i++) {
        const T* row = Cv.rows[A][i];
        T s2 = row[K] * f0;
        s2 += row[K + 1] * fN;
#pragma unroll
        for (int j = 0; j < K; j++) s2 += row[j] * v[j];
        q_elem[b0 + i * st] = s2;
    }
}

// Neighbour (or exterior) values of the two face nodes at the ends of line t
// along axis a, for the line owners above: drho always, the normal velocity
// with WITH_U, the gradient with WITH_Q (arrays not asked for are zeroed).
template <bool INCR, bool WITH_U, bool WITH_Q, typename T, int K>
__device__ __forceinline__ void line_end_values(const StageIO<T>& io, const MeshDev<T>& m,
                                                const OpConst<T, K>& C, int e, int a, int t, T ro[2], T uo[2],
                                                T qo[2])
{
    const int st = axis_stride<K>(a);
    const int b0 = a == 0 ? t : (a == 1 ? (t % K) * K * K + t / K : t * K);
#pragma unroll
    for (int side = 0; side < 2; side++) {
        ro[side] = T(0);
        uo[side] = T(0);
        qo[side] = T(0);
        const int code = __ldg(m.nbr + (size_t)e * 6 + 2 * a + side);
        if (code >= 0) {
            const size_t o2 = (size_t)code * io.np + b0 + (side ? 0 : (K - 1) * st);
            ro[side] = load_in<INCR>(io, 0, o2);
            if (WITH_U) uo[side] = load_in<INCR>(io, 1 + a, o2);
            if (WITH_Q) qo[side] = __ldg(io.q + (size_t)a * io.fs + o2);
        } else {
            T u2;
            exterior<T, K>(m, C, -1 - code, side, t, ro[side], u2);
            if (WITH_U) uo[side] = u2;
        }
    }
}

// Resident CTAs per SM asked of the compiler for the gradient kernel (0: no
// request): the FP32 kernel waits on memory latency and fits in 40 registers
// without spilling up to K = 5.
template <typename T, int K>
__host__ __device__ constexpr int grad_min_blocks()
{
    return (sizeof(T) == 4 && K <= 5) ? 65536 / (40 * npt_of(K) * epb_of(K)) : 0;
}

template <typename T, int K, bool INCR>
__global__ void __launch_bounds__(npt_of(K) * epb_of(K), (grad_min_blocks<T, K>()))
ldg_gradient_kernel(StageIO<T> io, MeshDev<T> m, const OpConst<T, K>* __restrict__ Cp, const OpConst<T, K> Cv)
{
    constexpr int K2 = K * K, K3 = K * K * K, NPT = npt_of(K), NF = 6 * K2, R = (NF + NPT - 1) / NPT;
    // FP32 (bound by the L1 data pipe) with K >= 5: line owners, as in
    // incr_stage_kernel; FP64 (bound by the FP64 pipe) keeps per-node sums.
    constexpr bool LINES = INCR && K >= 5;
    __shared__ GradSmem<T, K> sm_all[epb_of(K)];
    GradSmem<T, K>& S = sm_all[threadIdx.y];
    const OpConst<T, K>& C = *Cp;
    const int n = threadIdx.x;
    const int e = blockIdx.x * epb_of(K) + threadIdx.y;
    const bool live = e < m.n_elem;
    const bool act = n < K3 && live;
    const int c[3] = {n / K2, (n / K) % K, n % K};
    if constexpr (LINES) {
        // Line owners with their own face terms, storing their lines' results
        // themselves (every value of G has one owner): one barrier per element.
        constexpr int WPA = (K2 + 31) / 32;
        const int w = n / 32, a = w / WPA, t = (w % WPA) * 32 + n % 32;
        const bool owner = live && a < 3 && t < K2;
        T rho = T(0), ro[2] = {T(0), T(0)}, unused_u[2], unused_q[2];
        if (act) rho = load_in<INCR>(io, 0, (size_t)e * io.np + n);
        if (owner) line_end_values<INCR, false, false, T, K>(io, m, C, e, a, t, ro, unused_u, unused_q);
        S.r[n] = rho;
        __syncthreads();
        if (owner) {
            T* q = io.q_out + (size_t)a * io.fs + (size_t)e * io.np;
            if (a == 0) grad_line_faces<0>(Cv, S, t, ro, q);
            else if (a == 1) grad_line_faces<1>(Cv, S, t, ro, q);
            else grad_line_faces<2>(Cv, S, t, ro, q);
        }
    } else {
        // Face nodes assigned densely (see stage_kernel): their neighbour (or
        // exterior) values are loaded with the thread's own node.
        int code[R];
#pragma unroll
        for (int r = 0; r < R; r++) {
            const int t = n + r * NPT;
            code[r] = 0;
            if (live && t < NF) {
                const FaceNode<K> F(t);
                code[r] = __ldg(m.nbr + (size_t)e * 6 + 2 * F.a + F.side);
            }
        }
        T rho = T(0);
        if (act) rho = load_in<INCR>(io, 0, (size_t)e * io.np + n);
        T ro[R];
#pragma unroll
        for (int r = 0; r < R; r++) {
            ro[r] = T(0);
            const int t = n + r * NPT;
            if (!live || t >= NF) continue;
            const FaceNode<K> F(t);
            if (code[r] >= 0) {
                ro[r] = load_in<INCR>(io, 0, (size_t)code[r] * io.np + F.nn);
            } else {
                T uo;
                exterior<T, K>(m, C, -1 - code[r], F.side, F.fi, ro[r], uo);
            }
        }
        OpRows<T, K> R_;
        R_.load(C, c, act);
        S.r[n] = rho;
        __syncthreads();
#pragma unroll
        for (int r = 0; r < R; r++) {
            const int t = n + r * NPT;
            if (!live || t >= NF) continue;
            const FaceNode<K> F(t);
            S.fl[F.a][F.side][F.fi] = ro[r] + S.r[F.nf];  // flux factors are in the lift columns
        }
        __syncthreads();
        if (!act) return;
#pragma unroll
        for (int a = 0; a < 3; a++) {
            const int st = axis_stride<K>(a);
            const int base = n - c[a] * st;
            const int fi = c[(a + 1) % 3] * K + c[(a + 2) % 3];
            T s = R_.l0[a] * S.fl[a][0][fi];
            s += R_.ln[a] * S.fl[a][1][fi];
#pragma unroll
            for (int j = 0; j < K; j++) s += R_.d[a][j] * S.r[base + j * st];
            io.q_out[(size_t)a * io.fs + (size_t)e * io.np + n] = s;
        }
    }
}

// FP64 LDG gradient with even-odd line owners (K = 4, 5: eo_grad_lines): two
// elements per CTA so that the 3 K^2 line tasks of each pack densely into
// warps; each owner loads the neighbour values at its line's two ends, forms
// the central face sums, applies the even-odd operator and stores its line's
// K results of G_a itself (every value of G has exactly one owner), so the
// kernel has one barrier, after the element's values reach shared memory,
// and the threads without a line leave at it.  The stores along y- and
// z-lines are strided; the kernel is bound by the FP64 pipe, not by memory.
// Orders whose FP64 stage kernel uses even-odd line owners, by measurement on
// ~32.8 M nodes of config 2's physics (ms per launch, owners against per-node
// sums): K = 2: 8.99 / 11.71 (the per-node form leaves 24 of a warp slice's
// 32 lanes idle); K = 3: 4.49 / 4.57; K = 4: 3.891 / 3.845 (slower); K = 5:
// 3.85 / 4.12; K = 6 no faster (448-thread CTAs at 92 registers).
template <int K>
__host__ __device__ constexpr bool eo_lines()
{
    return K <= 3 || K == 5;
}

// The same choice for the gradient kernel (ms per launch): K = 2: 1.54 /
// 2.94; K = 3: 1.100 / 1.153; K = 4: 1.106 / 1.122; K = 5: 1.11 / 1.31;
// K = 6, 7, 8 slower (1.59 / 1.40, 1.73 / 1.60, 2.48 / 1.68).
template <int K>
__host__ __device__ constexpr bool eo_grad_lines()
{
    return K <= 5;
}

template <int K>
__device__ __forceinline__ void grad_eo_line(const LineEOAxis<K>& X, const GradSmem<double, K>& S, int a, int t,
                                             const double ro[2], double* __restrict__ q_elem)
{
    const int st = axis_stride<K>(a);
    const int b0 = a == 0 ? t : (a == 1 ? (t % K) * K * K + t / K : t * K);
    double v[K], out[K];
#pragma unroll
    for (int j = 0; j < K; j++) v[j] = S.r[b0 + j * st];
    eo_apply<K, -1>(X, v, ro[0] + v[0], ro[1] + v[K - 1], out);  // flux factors are in the lift columns
#pragma unroll
    for (int i = 0; i < K; i++) q_elem[b0 + i * st] = out[i];
}

template <int K>
__global__ void __launch_bounds__(npt_of(K) * 2)
ldg_gradient_eo_kernel(StageIO<double> io, MeshDev<double> m, const OpConst<double, K>* __restrict__ Cp,
                       const LineEO<K> L)
{
    constexpr int K2 = K * K, K3 = K2 * K, NPT = npt_of(K), EPB = 2, NL = 3 * K2;
    static_assert(NL <= NPT, "line tasks must fit the element's threads");
    __shared__ GradSmem<double, K> sm_all[EPB];
    __shared__ LineEOAxis<K> eo[3];
    const OpConst<double, K>& C = *Cp;
    const int n = threadIdx.x;
    const int e = blockIdx.x * EPB + threadIdx.y;
    const bool act = n < K3 && e < m.n_elem;
    if (threadIdx.y == 0 && n < 3) eo[n] = n == 0 ? L.ax[0] : (n == 1 ? L.ax[1] : L.ax[2]);
    // this thread's line task: element le of the CTA, axis la, line t
    const int tid = threadIdx.y * NPT + n;
    const int le = tid / NL, la = (tid % NL) / K2, t = tid % K2;
    const int el = blockIdx.x * EPB + le;
    const bool owner = tid < EPB * NL && el < m.n_elem;
    double rho = 0.0, ro[2] = {0.0, 0.0}, unused_u[2], unused_q[2];
    if (act) rho = __ldg(io.src + (size_t)e * io.np + n);
    if (owner) line_end_values<false, false, false, double, K>(io, m, C, el, la, t, ro, unused_u, unused_q);
    sm_all[threadIdx.y].r[n] = rho;
    __syncthreads();
    if (owner) grad_eo_line<K>(eo[la], sm_all[le], la, t, ro, io.q_out + (size_t)la * io.fs + (size_t)el * io.np);
}

// Shared memory of a stage kernel, per element: for each axis a, the pair
// (f_mom, f_mass along a + G_a) of every node (one 8- or 16-byte load feeds
// two FMAs of a line sum), the pair (momentum, density) of every face term
// [axis][side][face node], and each node's own mass flux and gradient, which
// the face phase reads (and the line owners then reuse for their results).
template <typename T, int K>
struct PlainSmem {
    typename Pair<T>::type f[3][npt_of(K)];
    typename Pair<T>::type g[3][2][K * K];
    T m[3][npt_of(K)];
    T q[3][npt_of(K)];
};

// ---------------------------------------------------------------------------
// One RK stage of the plain (FP64) form: R = L(stage input), then the stage
// combination dst = R' + s (cb - ca sigma) + cc old.
//
// The FP64 pipe is the bound, so the face fluxes are assigned densely: with
// per-node line sums, thread n of an element evaluates face nodes n, n + NPT,
// ... of its 6 K^2, reading the element's own values from shared memory; with
// even-odd line owners, each owner evaluates the two face nodes that end its
// line (the line tasks are packed densely too).  (A thread per node evaluating
// its own faces would issue every axis's face arithmetic in nearly every warp,
// since almost every warp holds some node on each face pair.)  The neighbour
// values of those face nodes are loaded with the thread's own node.
// ---------------------------------------------------------------------------
// Elements per CTA of the FP64 stage kernel: two with even-odd line owners
// (EO), so that the 3 K^2 line tasks of each pack densely into warps.
template <int K, bool EO>
__host__ __device__ constexpr int plain_epb()
{
    return EO ? 2 : epb_of(K);
}

// Resident CTAs per SM asked of the compiler for the FP64 stage kernel (0:
// no request): at K = 5, 64 registers keep 32 warps per SM.
template <typename T, int K, bool EO>
__host__ __device__ constexpr int plain_min_blocks()
{
    return (sizeof(T) == 8 && K == 5) ? 8 / plain_epb<K, EO>() : 0;
}

// One line of an FP64 stage kernel with even-odd line owners: the mass
// equation's line (flux f_mass + G, face terms gr) into S.m and the momentum
// equation's (f_mom, gm) into S.q, along runtime axis a.
// The line's face terms g0 (first node) and gN (last node) come from its
// owner (x momentum, y density).
template <int K>
__device__ __forceinline__ void stage_eo_line(const LineEOAxis<K>& X, PlainSmem<double, K>& S, int a, int t,
                                              int do_adv, const double2 g0, const double2 gN)
{
    const int st = axis_stride<K>(a);
    const int b0 = a == 0 ? t : (a == 1 ? (t % K) * K * K + t / K : t * K);
    // one field at a time (fewer live registers than both at once)
    double v[K], out[K];
#pragma unroll
    for (int j = 0; j < K; j++) v[j] = S.f[a][b0 + j * st].y;
    eo_apply<K, 1>(X, v, g0.y, gN.y, out);
#pragma unroll
    for (int i = 0; i < K; i++) S.m[a][b0 + i * st] = out[i];
    if (do_adv) {
#pragma unroll
        for (int j = 0; j < K; j++) v[j] = S.f[a][b0 + j * st].x;
        eo_apply<K, 1>(X, v, g0.x, gN.x, out);
#pragma unroll
        for (int i = 0; i < K; i++) S.q[a][b0 + i * st] = out[i];
    }
}

// Face term (x momentum, y density) of face node nf of an element on axis a,
// side ``side``: the numerical flux (impedance upwind for advection, central
// for LDG) times its lift scale, from the element's own values in shared
// memory and the neighbour (or exterior) values ro, uo (drho and the normal
// velocity, or in flux mode 2 their momentum and mass fluxes) and qo.
template <typename T, int K, bool DIFF, int FLUX>
__device__ __forceinline__ typename Pair<T>::type face_term(const OpConst<T, K>& C, const PlainSmem<T, K>& S,
                                                            int a, int side, int nf, T ro, T uo, T qo, int do_adv)
{
    const T fm_s = S.f[a][nf].x, fa_s = S.m[a][nf];
    T gm = T(0), gr = T(0);
    if (do_adv) {
        const T fmo = FLUX == 2 ? ro : momentum_flux(ro, C.k1, C.k2);
        const T fao = FLUX == 2 ? uo : mass_flux(uo, ro, C.r0, C.linear_mass);
        const T* cm = C.cM[a][side];
        const T* cr = C.cA[a][side];
        gm = fmo * cm[0] + fm_s * cm[1] + fao * cm[2] + fa_s * cm[3];
        gr = fmo * cr[0] + fm_s * cr[1] + fao * cr[2] + fa_s * cr[3];
    }
    if (DIFF) gr += C.cQ[a][side] * (qo + S.q[a][nf]);
    typename Pair<T>::type g;
    g.x = gm;
    g.y = gr;
    return g;
}

//
// Flux modes (FLUX; 1 and 2 only with advection on):
//   0: the volume fluxes of the element's nodes and of its face neighbours'
//      nodes are evaluated from the state;
//   1: as 0, and the fluxes of the output state are written to flux_out;
//   2: both are read from flux_in (the fluxes of src, written by the stage
//      that produced it) and those of the output are written to flux_out.
// Mode 2 trades 64 bytes of HBM traffic per node for the FP64 instructions
// of evaluating every interior face node's neighbour flux a second time
// (its own element evaluates it for its line sums).
//
// Line sums (EO): false, every node sums its three lines itself (operator
// rows in registers); true (D centro-antisymmetric, see LineEO), line owners
// apply the even-odd operator after the face phase, one more barrier, and
// each node adds its three axis results.
//
// PACK: the stage's output is also written in host order to io.pack (the
// last stage of a step whose result is downloaded: the pack rides on the
// FP64-bound stage instead of a kernel of its own).
template <typename T, int K, bool DIFF, int FLUX, bool EO, bool PACK = false>
__global__ void __launch_bounds__(npt_of(K) * plain_epb<K, EO>(), (plain_min_blocks<T, K, EO>()))
stage_kernel(StageIO<T> io, MeshDev<T> m, const OpConst<T, K>* __restrict__ Cp, const LineEO<K> L, int do_adv,
             int do_sponge)
{
    constexpr int K2 = K * K, K3 = K * K * K, NPT = npt_of(K), NF = 6 * K2, R = (NF + NPT - 1) / NPT;
    constexpr int EPB = plain_epb<K, EO>();
    __shared__ PlainSmem<T, K> sm_all[EPB];
    __shared__ LineEOAxis<K> eo[EO ? 3 : 1];
    PlainSmem<T, K>& S = sm_all[threadIdx.y];
    const OpConst<T, K>& C = *Cp;
    const int n = threadIdx.x;
    const int e = blockIdx.x * EPB + threadIdx.y;
    const bool live = e < m.n_elem;
    const bool act = n < K3 && live;
    const int c[3] = {n / K2, (n / K) % K, n % K};
    const size_t off = (size_t)e * io.np + n;
    OpRows<T, K> R_;
    if constexpr (EO) {
        if (threadIdx.y == 0 && n < 3) eo[n] = n == 0 ? L.ax[0] : (n == 1 ? L.ax[1] : L.ax[2]);
    } else {
        R_.load(C, c, act);
    }

    T rho = T(0), u[3] = {T(0), T(0), T(0)}, q[3] = {T(0), T(0), T(0)};
    T fl[4] = {T(0), T(0), T(0), T(0)};
    if (act) {
        if (FLUX != 2) {  // mode 2 needs the state only for the stage combination
            rho = load_in<false>(io, 0, off);
#pragma unroll
            for (int a = 0; a < 3; a++) u[a] = load_in<false>(io, 1 + a, off);
        }
        if (DIFF)
#pragma unroll
            for (int a = 0; a < 3; a++) q[a] = __ldg(io.q + (size_t)a * io.fs + off);
        if (FLUX == 2)
#pragma unroll
            for (int f = 0; f < 4; f++) fl[f] = __ldg(io.flux_in + (size_t)f * io.fs + off);
    }
    // Neighbour (or exterior) values of this thread's face nodes: drho and
    // the normal velocity, or in flux mode 2 their momentum and mass fluxes.
    // Per-node line sums: the element's 6 K^2 face nodes dealt out densely
    // (slots n, n + NPT, ...).  EO: the two ends of this thread's line task
    // (element le of the CTA, axis la, line lt), whose face terms its owner
    // evaluates itself, so the face phase needs no barrier of its own.
    constexpr int NL = 3 * K2, RF = EO ? 2 : R;
    const int tid = threadIdx.y * NPT + n;
    const int le = tid / NL, la = (tid % NL) / K2, lt = tid % K2;
    const bool owner = EO && tid < EPB * NL && blockIdx.x * EPB + le < m.n_elem;
    T ro[RF], uo[RF], qo[RF];
#pragma unroll
    for (int r = 0; r < RF; r++) {
        ro[r] = uo[r] = qo[r] = T(0);
        int fa, fside, ffi, fnn, fe;
        if constexpr (EO) {
            if (!owner) continue;
            const int st = axis_stride<K>(la);
            const int b0 = la == 0 ? lt : (la == 1 ? (lt % K) * K2 + lt / K : lt * K);
            fa = la;
            fside = r;
            ffi = lt;
            fnn = b0 + (r ? 0 : (K - 1) * st);
            fe = blockIdx.x * EPB + le;
        } else {
            const int t = n + r * NPT;
            if (!live || t >= NF) continue;
            const FaceNode<K> F(t);
            fa = F.a;
            fside = F.side;
            ffi = F.fi;
            fnn = F.nn;
            fe = e;
        }
        const int code = __ldg(m.nbr + (size_t)fe * 6 + 2 * fa + fside);
        if (code >= 0) {
            const size_t o2 = (size_t)code * io.np + fnn;
            if (FLUX == 2) {
                ro[r] = __ldg(io.flux_in + o2);
                uo[r] = __ldg(io.flux_in + (size_t)(1 + fa) * io.fs + o2);
            } else {
                ro[r] = load_in<false>(io, 0, o2);
                uo[r] = load_in<false>(io, 1 + fa, o2);
            }
            if (DIFF) qo[r] = __ldg(io.q + (size_t)fa * io.fs + o2);
        } else {
            exterior<T, K>(m, C, -1 - code, fside, ffi, ro[r], uo[r]);
            if (FLUX == 2) {
                const T fm = momentum_flux(ro[r], C.k1, C.k2);
                uo[r] = mass_flux(uo[r], ro[r], C.r0, C.linear_mass);
                ro[r] = fm;
            }
        }
    }

    T fmom = T(0), fmass[3] = {T(0), T(0), T(0)};
    if (FLUX == 2) {
        fmom = fl[0];
#pragma unroll
        for (int a = 0; a < 3; a++) fmass[a] = fl[1 + a];
    } else if (do_adv) {
        fmom = momentum_flux(rho, C.k1, C.k2);
#pragma unroll
        for (int a = 0; a < 3; a++) fmass[a] = mass_flux(u[a], rho, C.r0, C.linear_mass);
    }
#pragma unroll
    for (int a = 0; a < 3; a++) {
        S.f[a][n].x = fmom;
        S.f[a][n].y = DIFF ? fmass[a] + q[a] : fmass[a];
        S.m[a][n] = fmass[a];
        if (DIFF) S.q[a][n] = q[a];
    }
    __syncthreads();

    // Face terms (dense form): the numerical flux times its lift scale.
    if constexpr (!EO) {
#pragma unroll
        for (int r = 0; r < R; r++) {
            const int t = n + r * NPT;
            if (!live || t >= NF) continue;
            const FaceNode<K> F(t);
            S.g[F.a][F.side][F.fi] = face_term<T, K, DIFF, FLUX>(C, S, F.a, F.side, F.nf, ro[r], uo[r], qo[r], do_adv);
        }
        __syncthreads();
    }

    T r_rho = T(0), r_u[3] = {T(0), T(0), T(0)};
    if constexpr (EO) {
        static_assert(NL <= NPT, "line tasks must fit the element's threads");
        if (owner) {
            PlainSmem<T, K>& SL = sm_all[le];
            const int st = axis_stride<K>(la);
            const int b0 = la == 0 ? lt : (la == 1 ? (lt % K) * K2 + lt / K : lt * K);
            const typename Pair<T>::type g0 = face_term<T, K, DIFF, FLUX>(C, SL, la, 0, b0, ro[0], uo[0], qo[0], do_adv);
            const typename Pair<T>::type gN =
                face_term<T, K, DIFF, FLUX>(C, SL, la, 1, b0 + (K - 1) * st, ro[1], uo[1], qo[1], do_adv);
            stage_eo_line<K>(eo[la], SL, la, lt, do_adv, g0, gN);
        }
        __syncthreads();
        if (!act) return;
        r_rho = S.m[0][n] + S.m[1][n];
        r_rho += S.m[2][n];
#pragma unroll
        for (int a = 0; a < 3; a++) r_u[a] = do_adv ? S.q[a][n] : T(0);
    }
    if (!act) return;

    if constexpr (!EO) {
        // The density equation is one FMA chain through the three axes (no
        // per-axis partial sums to add): the kernel is bound by FP64 issue,
        // so every FP64 instruction saved per node counts.
#pragma unroll
        for (int a = 0; a < 3; a++) {
            const int st = axis_stride<K>(a), base = n - c[a] * st;
            const int fi = c[(a + 1) % 3] * K + c[(a + 2) % 3];
            const typename Pair<T>::type g0 = S.g[a][0][fi], gN = S.g[a][1][fi];
            T sm = R_.l0[a] * g0.x;
            sm += R_.ln[a] * gN.x;
            r_rho += R_.l0[a] * g0.y;
            r_rho += R_.ln[a] * gN.y;
#pragma unroll
            for (int j = 0; j < K; j++) {
                const typename Pair<T>::type v = S.f[a][base + j * st];
                sm += R_.d[a][j] * v.x;
                r_rho += R_.d[a][j] * v.y;
            }
            r_u[a] = do_adv ? sm : T(0);
        }
    }
    // cb - ca sigma of this element: tabulated per stage by the host, so that
    // no thread spends FP64 instructions on it; computed here when absent.
    const T cbe = io.elem_b ? __ldg(io.elem_b + e) : io.cb - (do_sponge ? io.ca * __ldg(m.sigma + e) : T(0));
    if (FLUX == 2) {
        rho = load_in<false>(io, 0, off);
#pragma unroll
        for (int a = 0; a < 3; a++) u[a] = load_in<false>(io, 1 + a, off);
    }

    const T r[4] = {r_rho, r_u[0], r_u[1], r_u[2]};
    const T s4[4] = {rho, u[0], u[1], u[2]};
    T vo[4];
#pragma unroll
    for (int f = 0; f < 4; f++) {
        const size_t o = (size_t)f * io.fs + off;
        T v = r[f] + s4[f] * cbe;
        if (io.old) v += io.old[o] * io.cc;
        io.dst[o] = v;
        vo[f] = v;
    }
    if (FLUX >= 1) {
        // the next stage's fluxes, evaluated as that stage would from dst
        io.flux_out[off] = momentum_flux(vo[0], C.k1, C.k2);
#pragma unroll
        for (int a = 0; a < 3; a++)
            io.flux_out[(size_t)(1 + a) * io.fs + off] = mass_flux(vo[1 + a], vo[0], C.r0, C.linear_mass);
    }
    if constexpr (PACK) {
        const size_t gi = grid_index(io.pack_map, e, n);
#pragma unroll
        for (int f = 0; f < 4; f++) io.pack[(size_t)f * io.pack_gsize + gi] = (double)vo[f];
    }
}

// ---------------------------------------------------------------------------
// One RK stage of the increment (FP32) form.  The kernel waits on memory
// latency and on the L1 data pipe, so every global load a thread makes is
// issued before the first value is used (face-table codes and sigma, its own
// u, d, gradient and Kahan compensation, the neighbour values of its face
// nodes), and the face nodes are assigned densely as in stage_kernel, which
// also makes the neighbour gathers denser warp requests.  The face fluxes are
// evaluated after a barrier from the element's own values in shared memory.
//
// The line sums (the L1 data pipe's largest load: 2 (K + 2) shared-memory
// operands per node and axis when each node sums its own lines) are done by
// line owners for K >= 5: warps take one axis each, a lane one line of the
// element, reads the line's K flux pairs and two face terms once and produces
// all K outputs, with the operator rows taken from kernel-parameter space
// (``Cv``; warp-uniform indices, so constant-bank operands).  The per-axis
// results go to shared memory and each node thread adds them up.
// ---------------------------------------------------------------------------
// Resident CTAs per SM asked of the compiler for the FP32 stage kernel (0: no
// request): at K = 5 it fits 40 registers without spilling, 12 CTAs per SM.
template <typename T, int K>
__host__ __device__ constexpr int incr_min_blocks()
{
    return (sizeof(T) == 4 && K == 5) ? 12 : 0;
}

template <typename T, int K, bool DIFF>
__global__ void __launch_bounds__(npt_of(K) * epb_of(K), (incr_min_blocks<T, K>()))
incr_stage_kernel(StageIO<T> io, MeshDev<T> m, const OpConst<T, K>* __restrict__ Cp, const OpConst<T, K> Cv,
                  int do_adv, int do_sponge)
{
    constexpr bool LINES = K >= 5;  // three warp-groups of ceil(K^2 / 32) warps fit in NPT
    constexpr int K2 = K * K, K3 = K * K * K, NPT = npt_of(K), NF = 6 * K2, R = (NF + NPT - 1) / NPT;
    constexpr int WPA = (K2 + 31) / 32;
    __shared__ PlainSmem<T, K> sm_all[epb_of(K)];
    PlainSmem<T, K>& S = sm_all[threadIdx.y];
    const OpConst<T, K>& C = *Cp;
    const int n = threadIdx.x;
    const int e = blockIdx.x * epb_of(K) + threadIdx.y;
    const bool live = e < m.n_elem;
    const bool act = n < K3 && live;
    const int c[3] = {n / K2, (n / K) % K, n % K};
    const size_t off = (size_t)e * io.np + n;
    // line owner (LINES): warp group a, line t of that axis
    const int la = n / 32 / WPA, lt = (n / 32 % WPA) * 32 + n % 32;
    const bool owner = LINES && live && la < 3 && lt < K2;

    int code[R];
    if constexpr (!LINES) {
#pragma unroll
        for (int r = 0; r < R; r++) {
            const int t = n + r * NPT;
            code[r] = 0;
            if (live && t < NF) {
                const FaceNode<K> F(t);
                code[r] = __ldg(m.nbr + (size_t)e * 6 + 2 * F.a + F.side);
            }
        }
    }
    const T sig = (act && do_sponge) ? __ldg(m.sigma + e) : T(0);
    T ub[4] = {T(0), T(0), T(0), T(0)}, dv[4] = {T(0), T(0), T(0), T(0)};
    T cmp[4] = {T(0), T(0), T(0), T(0)}, q[3] = {T(0), T(0), T(0)};
    if (act) {
#pragma unroll
        for (int f = 0; f < 4; f++) {
            ub[f] = __ldg(io.src + (size_t)f * io.fs + off);
            if (io.inc) dv[f] = __ldg(io.inc + (size_t)f * io.fs + off);
            if (io.final_stage) cmp[f] = io.comp[(size_t)f * io.fs + off];
        }
        if (DIFF)
#pragma unroll
            for (int a = 0; a < 3; a++) q[a] = __ldg(io.q + (size_t)a * io.fs + off);
    }
    // Neighbour (or exterior) values: of the two ends of the owned line
    // (LINES), else of the densely assigned face nodes.
    T ro[R > 2 ? R : 2], uo[R > 2 ? R : 2], qo[R > 2 ? R : 2];
    if constexpr (LINES) {
        if (owner) line_end_values<true, true, DIFF, T, K>(io, m, C, e, la, lt, ro, uo, qo);
    } else {
#pragma unroll
        for (int r = 0; r < R; r++) {
            ro[r] = uo[r] = qo[r] = T(0);
            const int t = n + r * NPT;
            if (!live || t >= NF) continue;
            const FaceNode<K> F(t);
            if (code[r] >= 0) {
                const size_t o2 = (size_t)code[r] * io.np + F.nn;
                ro[r] = load_in<true>(io, 0, o2);
                uo[r] = load_in<true>(io, 1 + F.a, o2);
                if (DIFF) qo[r] = __ldg(io.q + (size_t)F.a * io.fs + o2);
            } else {
                exterior<T, K>(m, C, -1 - code[r], F.side, F.fi, ro[r], uo[r]);
            }
        }
    }
    OpRows<T, K> R_;
    if constexpr (!LINES) R_.load(C, c, act);

    const T rho = ub[0] + dv[0];
    const T u[3] = {ub[1] + dv[1], ub[2] + dv[2], ub[3] + dv[3]};
    T fmom = T(0), fmass[3] = {T(0), T(0), T(0)};
    if (do_adv) {
        fmom = momentum_flux(rho, C.k1, C.k2);
#pragma unroll
        for (int a = 0; a < 3; a++) fmass[a] = mass_flux(u[a], rho, C.r0, C.linear_mass);
    }
#pragma unroll
    for (int a = 0; a < 3; a++) {
        S.f[a][n].x = fmom;
        S.f[a][n].y = DIFF ? fmass[a] + q[a] : fmass[a];
        S.m[a][n] = fmass[a];
        if (DIFF) S.q[a][n] = q[a];
    }
    __syncthreads();

    T r[4] = {T(0), T(0), T(0), T(0)};
    if constexpr (LINES) {
        // Line owners evaluate the face terms at both ends of their line and
        // the line sums; the per-axis results reuse S.m (density) and S.q
        // (momentum) of the owner's own line nodes, read before written.
        if (owner) {
            if (la == 0) stage_line_faces<0, DIFF>(Cv, S, lt, ro, uo, qo, do_adv);
            else if (la == 1) stage_line_faces<1, DIFF>(Cv, S, lt, ro, uo, qo, do_adv);
            else stage_line_faces<2, DIFF>(Cv, S, lt, ro, uo, qo, do_adv);
        }
        __syncthreads();
        if (!act) return;
#pragma unroll
        for (int a2 = 0; a2 < 3; a2++) {
            r[0] += S.m[a2][n];
            r[1 + a2] = do_adv ? S.q[a2][n] : T(0);
        }
    } else {
#pragma unroll
        for (int rr = 0; rr < R; rr++) {
            const int t = n + rr * NPT;
            if (!live || t >= NF) continue;
            const FaceNode<K> F(t);
            const T fm_s = S.f[F.a][F.nf].x, fa_s = S.m[F.a][F.nf];
            T gm = T(0), gr = T(0);
            if (do_adv) {
                const T fmo = momentum_flux(ro[rr], C.k1, C.k2);
                const T fao = mass_flux(uo[rr], ro[rr], C.r0, C.linear_mass);
                const T* cm = C.cM[F.a][F.side];
                const T* cr = C.cA[F.a][F.side];
                gm = fmo * cm[0] + fm_s * cm[1] + fao * cm[2] + fa_s * cm[3];
                gr = fmo * cr[0] + fm_s * cr[1] + fao * cr[2] + fa_s * cr[3];
            }
            if (DIFF) gr += C.cQ[F.a][F.side] * (qo[rr] + S.q[F.a][F.nf]);
            S.g[F.a][F.side][F.fi].x = gm;
            S.g[F.a][F.side][F.fi].y = gr;
        }
        __syncthreads();
        if (!act) return;
#pragma unroll
        for (int a = 0; a < 3; a++) {
            const int st = axis_stride<K>(a), base = n - c[a] * st;
            const int fi = c[(a + 1) % 3] * K + c[(a + 2) % 3];
            const typename Pair<T>::type g0 = S.g[a][0][fi], gN = S.g[a][1][fi];
            T sm = R_.l0[a] * g0.x, sr = R_.l0[a] * g0.y;
            sm += R_.ln[a] * gN.x;
            sr += R_.ln[a] * gN.y;
#pragma unroll
            for (int j = 0; j < K; j++) {
                const typename Pair<T>::type v = S.f[a][base + j * st];
                sm += R_.d[a][j] * v.x;
                sr += R_.d[a][j] * v.y;
            }
            r[0] += sr;
            r[1 + a] = do_adv ? sm : T(0);
        }
    }
    const T ks = io.ca * sig;
    const T cbe = io.cb - ks, ce = io.eps - ks;
#pragma unroll
    for (int f = 0; f < 4; f++) {
        const size_t o = (size_t)f * io.fs + off;
        T d = r[f] + ub[f] * ce;
        if (io.inc) d += dv[f] * cbe;
        if (io.final_stage) {
            // Kahan-compensated u <- u + d
            const T y = d - cmp[f];
            const T t = ub[f] + y;
            io.comp[o] = (t - ub[f]) - y;
            io.dst[o] = t;
        } else {
            io.dst[o] = d;
        }
    }
}

// Host-side construction of the per-launch operators from the FP64 line
// operators (M^-1 S, lift columns) and the problem constants.
// ``rk_ca`` is the stage weight of R (1 for a bare right-hand side).
template <typename T, int K>
inline OpConst<T, K> make_stage_const(double rk_ca, const double* deriv, const double* lift0, const double* liftN,
                                      const double w[3], double rho0, double c0, double b_over_a,
                                      double diff_const)
{
    OpConst<T, K> C{};
    for (int a = 0; a < 3; a++)
        for (int i = 0; i < K; i++) {
            C.rows[a][i][K] = (T)lift0[i];
            C.rows[a][i][K + 1] = (T)liftN[i];
        }
    // Face-flux coefficients as the reference forms them (cppsrc/Element.cpp:542-556
    // left, :581-595 right); z = rho0 c0 and r = rho0 on both sides.
    const double r0 = rho0, z1 = r0 * c0, z2 = r0 * c0, r1 = r0, r2 = r0;
    const double cL0[4] = {z1 * r2 / (z1 + z2), z2 * r1 / (z1 + z2), z1 * z2 / r2 / (z1 + z2),
                           -1.0 * z1 * z2 / r1 / (z1 + z2)};
    const double cL1[4] = {z2 / r2 / (z1 + z2), z1 / r1 / (z1 + z2), r2 / (z1 + z2), -1.0 * r1 / (z1 + z2)};
    const double cR0[4] = {z2 * r1 / (z1 + z2), z1 * r2 / (z1 + z2), z1 * z2 / r1 / (z1 + z2),
                           -1.0 * z1 * z2 / r2 / (z1 + z2)};
    const double cR1[4] = {z1 / r1 / (z1 + z2), z2 / r2 / (z1 + z2), r1 / (z1 + z2), -1.0 * r2 / (z1 + z2)};
    for (int a = 0; a < 3; a++) {
        for (int i = 0; i < K; i++)
            for (int j = 0; j < K; j++) C.rows[a][i][j] = (T)(rk_ca * deriv[i * K + j] / w[a]);
        // momentum: lift scale -1/(rho0 w); left flux F_0 = -(fmo cL0[0] + fms cL0[1]
        // + fao cL0[2] + fas cL0[3]), right F_N = fms cR0[0] + fmo cR0[1] + fas cR0[2] + fao cR0[3]
        const double km = rk_ca * (-1.0 / (r0 * w[a]));
        const double lm[4] = {-cL0[0], -cL0[1], -cL0[2], -cL0[3]};
        const double rm[4] = {cR0[1], cR0[0], cR0[3], cR0[2]};
        // mass: lift scale -rho0/w; left F_0 = -(fao cL1[0] + fas cL1[1] + fmo cL1[2] + fms cL1[3]),
        // right F_N = fas cR1[0] + fao cR1[1] + fms cR1[2] + fmo cR1[3]
        const double ka = rk_ca * (-r0 / w[a]);
        const double la[4] = {-cL1[2], -cL1[3], -cL1[0], -cL1[1]};
        const double ra[4] = {cR1[3], cR1[2], cR1[1], cR1[0]};
        for (int i = 0; i < 4; i++) {
            C.cM[a][0][i] = (T)(km * lm[i]);
            C.cM[a][1][i] = (T)(km * rm[i]);
            C.cA[a][0][i] = (T)(ka * la[i]);
            C.cA[a][1][i] = (T)(ka * ra[i]);
        }
        // LDG divergence of G = -D_c Q: (1/w)(D G + lift(central flux of G))
        C.cQ[a][0] = (T)(0.5 * rk_ca / w[a]);
        C.cQ[a][1] = (T)(-0.5 * rk_ca / w[a]);
    }
    const FluxOut<T> fc = flux_consts<T>(nullptr, r0, c0, b_over_a);
    C.k1 = fc.k1;
    C.k2 = fc.k2;
    C.r0 = fc.r0;
    C.inv_c2 = (T)(1.0 / (c0 * c0));
    C.inv_z = (T)(1.0 / (r0 * c0));
    C.linear_mass = fc.linear;
    (void)diff_const;
    return C;
}

template <typename T, int K>
inline OpConst<T, K> make_grad_const(const double* deriv, const double* lift0, const double* liftN,
                                     const double w[3], double rho0, double c0, double diff_const)
{
    OpConst<T, K> C{};
    for (int a = 0; a < 3; a++) {
        // central flux of drho, (+0.5, -0.5) D_c / w_a, folded into the lift
        // columns: the kernels lift the plain face sum (own + other)
        const double q0 = 0.5 * diff_const / w[a], qN = -0.5 * diff_const / w[a];
        for (int i = 0; i < K; i++) {
            for (int j = 0; j < K; j++) C.rows[a][i][j] = (T)(diff_const * deriv[i * K + j] / w[a]);
            C.rows[a][i][K] = (T)(lift0[i] * q0);
            C.rows[a][i][K + 1] = (T)(liftN[i] * qN);
        }
        C.cQ[a][0] = C.cQ[a][1] = T(1);
    }
    C.inv_c2 = (T)(1.0 / (c0 * c0));
    C.inv_z = (T)(1.0 / (rho0 * c0));
    return C;
}

// Even-odd split of the per-axis rows of C (see LineEO); false when D is not
// centro-antisymmetric or the lift columns are not mirrored with sign SIG, to
// 1e-12 of their largest entry, and the line owners must not be used.
template <int K, int SIG>
inline bool make_line_eo(const OpConst<double, K>& C, LineEO<K>& L)
{
    constexpr int H = K / 2;
    if (H < 1) return false;
    for (int a = 0; a < 3; a++) {
        const auto& R = C.rows[a];
        double dmax = 0.0, lmax = 0.0;
        for (int i = 0; i < K; i++) {
            for (int j = 0; j < K; j++) dmax = std::fmax(dmax, std::fabs(R[i][j]));
            lmax = std::fmax(lmax, std::fmax(std::fabs(R[i][K]), std::fabs(R[i][K + 1])));
        }
        for (int i = 0; i < K; i++) {
            for (int j = 0; j < K; j++)
                if (std::fabs(R[i][j] + R[K - 1 - i][K - 1 - j]) > 1e-12 * dmax) return false;
            if (std::fabs(R[K - 1 - i][K] - SIG * R[i][K + 1]) > 1e-12 * lmax) return false;
        }
        for (int i = 0; i < H; i++) {
            for (int j = 0; j < H; j++) {
                L.ax[a].E[i][j] = 0.5 * (R[i][j] + R[i][K - 1 - j]);
                L.ax[a].O[i][j] = 0.5 * (R[i][j] - R[i][K - 1 - j]);
            }
            L.ax[a].Dc[i] = (K & 1) ? R[i][H] : 0.0;
            L.ax[a].Al[i] = 0.5 * (R[i][K] + R[i][K + 1]);
            L.ax[a].Bl[i] = 0.5 * (R[i][K] - R[i][K + 1]);
            L.ax[a].Dm[i] = (K & 1) ? R[H][i] : 0.0;
        }
        L.ax[a].Lm = (K & 1) ? R[H][K] : 0.0;
    }
    return true;
}

// State <-> host-order arrays rho [X][Y][Z], vel [3][X][Y][Z], walked in host
// order so that rho/vel may be pinned host memory read or written directly by
// the kernel (streaming, coalesced on the host side), or device staging.  A
// CTA takes one (x, y) row at a time and its threads walk z, so the element
// arithmetic is 32-bit and mostly per row.
struct RowMap {
    int elem_xy;  // element-index part of the row's element coordinates
    int node_xy;  // (a K + b) K: node-index part of the row
};

__device__ __forceinline__ RowMap row_map(const GridMap& g, int ii, int jj)
{
    const int K = g.K;
    const int gx = ii / K, gy = jj / K;
    const int bx = gx / g.ne[0], by = gy / g.ne[1], lx = gx % g.ne[0], ly = gy % g.ne[1];
    return {(bx * g.nb[1] + by) * g.nb[2] * g.elem_per_block + (lx * g.ne[1] + ly) * g.ne[2],
            ((ii % K) * K + jj % K) * K};
}

__device__ __forceinline__ size_t row_offset(const GridMap& g, int np, const RowMap& r, int kk)
{
    const int gz = kk / g.K;
    const int e = r.elem_xy + (gz / g.ne[2]) * g.elem_per_block + gz % g.ne[2];
    return (size_t)e * np + r.node_xy + kk % g.K;
}

template <typename T>
__global__ void pack_host_order_kernel(const T* __restrict__ state, size_t fs, int np, GridMap g,
                                       double* __restrict__ rho, double* __restrict__ vel, size_t gsize)
{
    const int Y = g.E[1] * g.K, Z = g.E[2] * g.K, rows = g.E[0] * g.K * Y;
    for (int row = blockIdx.x; row < rows; row += gridDim.x) {
        const RowMap r = row_map(g, row / Y, row % Y);
        for (int kk = threadIdx.x; kk < Z; kk += blockDim.x) {
            const size_t o = row_offset(g, np, r, kk), i = (size_t)row * Z + kk;
            if (rho) rho[i] = (double)state[o];
            if (vel)
#pragma unroll
                for (int a = 0; a < 3; a++) vel[a * gsize + i] = (double)state[(size_t)(1 + a) * fs + o];
        }
    }
}

template <typename T>
__global__ void unpack_host_order_kernel(T* __restrict__ state, size_t fs, int np, GridMap g,
                                         const double* __restrict__ rho, const double* __restrict__ vel, size_t gsize,
                                         FluxOut<T> fo)
{
    const int Y = g.E[1] * g.K, Z = g.E[2] * g.K, rows = g.E[0] * g.K * Y;
    for (int row = blockIdx.x; row < rows; row += gridDim.x) {
        const RowMap r = row_map(g, row / Y, row % Y);
        for (int kk = threadIdx.x; kk < Z; kk += blockDim.x) {
            const size_t o = row_offset(g, np, r, kk), i = (size_t)row * Z + kk;
            const T d = (T)rho[i];
            T u[3];
            state[o] = d;
#pragma unroll
            for (int a = 0; a < 3; a++) {
                u[a] = (T)vel[a * gsize + i];
                state[(size_t)(1 + a) * fs + o] = u[a];
            }
            if (fo.f) write_fluxes(fo, fs, o, d, u);
        }
    }
}

// Host-order device staging -> state, walked in element order: the state
// writes are contiguous per element and the scattered side is the read
// (K-value runs along z), which costs less than partial-sector writes.  For
// device memory only; pinned host memory is read by unpack_host_order_kernel.
template <typename T>
__global__ void unpack_elem_order_kernel(T* __restrict__ state, size_t fs, int np, GridMap g, int n_elem,
                                         const double* __restrict__ rho, const double* __restrict__ vel, size_t gsize,
                                         FluxOut<T> fo)
{
    const int K3 = g.K * g.K * g.K;
    const size_t total = (size_t)n_elem * np;
    for (size_t s = blockIdx.x * (size_t)blockDim.x + threadIdx.x; s < total; s += (size_t)gridDim.x * blockDim.x) {
        const int e = (int)(s / np), n = (int)(s % np);
        if (n >= K3) continue;
        const size_t i = grid_index(g, e, n);
        const T d = (T)rho[i];
        T u[3];
        state[s] = d;
#pragma unroll
        for (int a = 0; a < 3; a++) {
            u[a] = (T)vel[a * gsize + i];
            state[(size_t)(1 + a) * fs + s] = u[a];
        }
        if (fo.f) write_fluxes(fo, fs, s, d, u);
    }
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


}  // namespace dg
