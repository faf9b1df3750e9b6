// dg_eval_rhs_noalloc: the right-hand-side evaluation of dg_eval_rhs for
// callers that cannot allocate device memory.
//
// Who needs it: code that runs where cudaMalloc is not allowed or not wanted
// at call time — a host that owns all device memory through its own pool or
// a fixed arena (simulation frameworks, embedded real-time loops), or code that
// must not add allocations to a process whose memory is budgeted.  Such a
// caller cannot create a dg_handle (dg_create allocates the state, stage and
// gradient buffers); it already holds the state and the mesh tables in memory
// it owns and only needs R = L(u) computed.
//
// The one scratch this computation needs, the LDG gradient Q (3 fields per
// node), lives in a file-scope static device array instead of an allocation:
// every GPU that loads this library holds it (27 MiB) until the process exits.
// Its device address is looked up once per device with cudaGetSymbolAddress
// (host code cannot use the array's name as a device address).  With CUDA's
// default lazy module loading that first look-up also loads this file's
// device code on the device, and the 27 MiB is taken then: a host that
// budgets device memory makes one call per device at start-up, before it
// commits its own arena.  The address is cached for the life of the process,
// so a cudaDeviceReset of a device invalidates it (this entry point is not
// for processes that reset devices while it is loaded).  Every call shares the
// array and it keeps the last call's contents: the gradient part is fully
// rewritten by each call before it is read, the boundary-flag part is cleared
// by each call, the operator part is rewritten by each call, and calls whose
// work overlaps on the same GPU (for example calls issued to two streams with
// no ordering between them) race on it.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <mutex>
#include <string>

#include "dg3d.h"
#include "dg_kernels.cuh"
#include "solver_internal.h"

namespace {

constexpr size_t kMaxSlots = DG_NOALLOC_MAX_NODES;    // n_elem * NP, padded node slots
constexpr size_t kMaxElems = DG_NOALLOC_MAX_ELEMENTS;
constexpr size_t kQBytes = 3 * kMaxSlots * sizeof(double);
constexpr size_t kFlagBytes = 6 * kMaxElems * sizeof(int);
constexpr size_t kConstSlot = 4096;  // one per-launch operator (OpConst<double, 8> fits)

// LDG gradient (3 x kMaxSlots doubles), the boundary-source flags (6 x
// kMaxElems ints, zero: every boundary face reads a zero exterior state) and
// two operator slots (stage, gradient).
static __device__ __align__(256) unsigned char g_noalloc_scratch[kQBytes + kFlagBytes + 2 * kConstSlot];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
void* g_scratch_addr[kMaxDevices] = {};

// Set-up, once per device, with that device current.
int scratch_address(void** out)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return dg::fail(DG_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    if (dev < 0 || dev >= kMaxDevices) return dg::fail(DG_ERR_INVALID, "dg_eval_rhs_noalloc: device index too large");
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_addr[dev]) {
        void* ptr = nullptr;
        e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
        if (e != cudaSuccess || !ptr)
            return dg::fail(DG_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
        g_scratch_addr[dev] = ptr;
    }
    *out = g_scratch_addr[dev];
    return DG_OK;
}

// D = M^-1 S and the lift columns M^-1 e_0, M^-1 e_N, on the stack.
bool line_operators_stack(int K, const double* M, const double* S, double* D, double* L0, double* LN)
{
    double A[64], B[64 + 16];
    const int R = K + 2;
    for (int i = 0; i < K * K; i++) A[i] = M[i];
    for (int i = 0; i < K; i++) {
        for (int j = 0; j < K; j++) B[i * R + j] = S[i * K + j];
        B[i * R + K] = i == 0 ? 1.0 : 0.0;
        B[i * R + K + 1] = i == K - 1 ? 1.0 : 0.0;
    }
    for (int c = 0; c < K; c++) {
        int piv = c;
        for (int i = c + 1; i < K; i++)
            if (std::fabs(A[i * K + c]) > std::fabs(A[piv * K + c])) piv = i;
        if (A[piv * K + c] == 0.0) return false;
        if (piv != c) {
            for (int j = 0; j < K; j++) std::swap(A[c * K + j], A[piv * K + j]);
            for (int r = 0; r < R; r++) std::swap(B[c * R + r], B[piv * R + r]);
        }
        for (int i = c + 1; i < K; i++) {
            const double m = A[i * K + c] / A[c * K + c];
            for (int j = c; j < K; j++) A[i * K + j] -= m * A[c * K + j];
            for (int r = 0; r < R; r++) B[i * R + r] -= m * B[c * R + r];
        }
    }
    for (int r = 0; r < R; r++)
        for (int i = K - 1; i >= 0; i--) {
            double v = B[i * R + r];
            for (int j = i + 1; j < K; j++) v -= A[i * K + j] * B[j * R + r];
            B[i * R + r] = v / A[i * K + i];
        }
    for (int i = 0; i < K; i++) {
        for (int j = 0; j < K; j++) D[i * K + j] = B[i * R + j];
        L0[i] = B[i * R + K];
        LN[i] = B[i * R + K + 1];
    }
    return true;
}

// Writes the two per-launch operator blocks into the scratch.  They travel as
// kernel arguments, which the launch copies, so nothing is read from the
// caller's host stack after this function returns.
template <int K>
__global__ void store_operators_kernel(dg::OpConst<double, K>* __restrict__ dst, const dg::OpConst<double, K> C,
                                       const dg::OpConst<double, K> G)
{
    static_assert(sizeof(dg::OpConst<double, K>) % sizeof(int) == 0, "operator block size");
    constexpr int NW = (int)(sizeof(dg::OpConst<double, K>) / sizeof(int));
    const int* c = reinterpret_cast<const int*>(&C);
    const int* g = reinterpret_cast<const int*>(&G);
    int* d0 = reinterpret_cast<int*>(dst);
    int* d1 = reinterpret_cast<int*>(reinterpret_cast<unsigned char*>(dst) + kConstSlot);
    for (int i = threadIdx.x; i < NW; i += blockDim.x) {
        d0[i] = c[i];
        d1[i] = g[i];
    }
}

template <int K>
cudaError_t launch(const dg_params& p, const double* D, const double* L0, const double* LN,
                   const dg::StageIO<double>& io, const dg::MeshDev<double>& md, unsigned char* consts,
                   cudaStream_t st)
{
    static_assert(sizeof(dg::OpConst<double, K>) <= kConstSlot, "operator slot too small");
    const dg::OpConst<double, K> C = dg::make_stage_const<double, K>(1.0, D, L0, LN, p.elem_width, p.rho0, p.c0,
                                                                     p.b_over_a, p.diff_const);
    const dg::OpConst<double, K> G =
        dg::make_grad_const<double, K>(D, L0, LN, p.elem_width, p.rho0, p.c0, p.diff_const);
    store_operators_kernel<K><<<1, 128, 0, st>>>((dg::OpConst<double, K>*)consts, C, G);
    const dg::OpConst<double, K>* Cd = (const dg::OpConst<double, K>*)consts;
    const dg::OpConst<double, K>* Gd = (const dg::OpConst<double, K>*)(consts + kConstSlot);
    dim3 block(dg::npt_of(K), dg::epb_of(K));
    dim3 grid((md.n_elem + dg::epb_of(K) - 1) / dg::epb_of(K));
    if (p.eval_diff) {
        dg::ldg_gradient_kernel<double, K, false><<<grid, block, 0, st>>>(io, md, Gd, G);
        dg::stage_kernel<double, K, true, 0, false><<<grid, block, 0, st>>>(io, md, Cd, dg::LineEO<K>{}, p.eval_advect,
                                                                          p.eval_sponge);
    } else {
        dg::stage_kernel<double, K, false, 0, false><<<grid, block, 0, st>>>(io, md, Cd, dg::LineEO<K>{}, p.eval_advect,
                                                                          p.eval_sponge);
    }
    return cudaSuccess;
}

}  // namespace

extern "C" int dg_eval_rhs_noalloc(const dg_params* p, const double* mass, const double* stiff,
                                   const double* d_state, const int* d_nbr, const double* d_sigma,
                                   double* d_rhs, int n_elem, void* stream)
{
    if (!p || !mass || !stiff || !d_state || !d_nbr || !d_rhs || (p->eval_sponge && !d_sigma))
        return dg::fail(DG_ERR_INVALID, "dg_eval_rhs_noalloc: null argument");
    if (p->precision != DG_PRECISION_FP64)
        return dg::fail(DG_ERR_INVALID, "dg_eval_rhs_noalloc: FP64 only");
    if (p->order < 1 || p->order > 7) return dg::fail(DG_ERR_INVALID, "dg_eval_rhs_noalloc: ORDER must be in 1..7");
    if (!(p->rho0 > 0.0) || !(p->c0 > 0.0)) return dg::fail(DG_ERR_INVALID, "dg_eval_rhs_noalloc: bad medium");
    const int K = p->order + 1;
    const long long np = (K * K * K + 7) / 8 * 8;
    if (n_elem < 1) return dg::fail(DG_ERR_INVALID, "dg_eval_rhs_noalloc: n_elem must be >= 1");
    if ((unsigned long long)n_elem > kMaxElems || (unsigned long long)(n_elem * np) > kMaxSlots)
        return dg::fail(DG_ERR_INVALID,
                        "dg_eval_rhs_noalloc: problem too large for the static scratch: n_elem = " +
                            std::to_string(n_elem) + " with " + std::to_string(np) +
                            " node slots per element exceeds the maximum of " + std::to_string(kMaxElems) +
                            " elements and " + std::to_string(kMaxSlots) + " node slots");
    double D[64], L0[8], LN[8];
    if (!line_operators_stack(K, mass, stiff, D, L0, LN))
        return dg::fail(DG_ERR_INVALID, "dg_eval_rhs_noalloc: mass matrix is singular");
    void* scratch = nullptr;
    int rc = scratch_address(&scratch);
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    double* q = (double*)scratch;
    int* flags = (int*)((unsigned char*)scratch + kQBytes);
    unsigned char* consts = (unsigned char*)scratch + kQBytes + kFlagBytes;
    cudaError_t e = cudaMemsetAsync(flags, 0, (size_t)6 * n_elem * sizeof(int), st);
    if (e != cudaSuccess) return dg::fail(DG_ERR_CUDA, std::string("cudaMemsetAsync: ") + cudaGetErrorString(e));

    dg::StageIO<double> io;
    std::memset(&io, 0, sizeof io);
    io.src = d_state;
    io.dst = d_rhs;
    io.q = q;
    io.q_out = q;
    io.fs = (size_t)n_elem * np;
    io.np = (int)np;
    io.ca = 1.0;
    io.cb = 0.0;
    dg::MeshDev<double> md;
    md.nbr = d_nbr;
    md.sigma = d_sigma;
    md.bnd_ic = nullptr;
    md.bnd_ap = nullptr;
    md.bnd_src = flags;
    md.n_elem = n_elem;
    md.ic_live = 0;
    md.src_p = 0.0;
    switch (K) {
    case 2: e = launch<2>(*p, D, L0, LN, io, md, consts, st); break;
    case 3: e = launch<3>(*p, D, L0, LN, io, md, consts, st); break;
    case 4: e = launch<4>(*p, D, L0, LN, io, md, consts, st); break;
    case 5: e = launch<5>(*p, D, L0, LN, io, md, consts, st); break;
    case 6: e = launch<6>(*p, D, L0, LN, io, md, consts, st); break;
    case 7: e = launch<7>(*p, D, L0, LN, io, md, consts, st); break;
    case 8: e = launch<8>(*p, D, L0, LN, io, md, consts, st); break;
    }
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e != cudaSuccess) return dg::fail(DG_ERR_CUDA, std::string("kernel launch: ") + cudaGetErrorString(e));
    return DG_OK;
}
