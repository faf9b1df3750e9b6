// libdg3d: the C ABI of include/dg3d.h.  Owns the device buffers of one
// simulation, issues the stage kernels of dg_kernels.cuh on its own stream and
// moves state between host and device only on request.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "basis.h"
#include "dg3d.h"
#include "dg_kernels.cuh"
#include "mesh.h"
#include "solver_internal.h"

namespace dg {

thread_local std::string g_last_error;

int fail(int code, const std::string& msg)
{
    g_last_error = msg;
    return code;
}

#define DG_CUDA(call)                                                                          \
    do {                                                                                       \
        cudaError_t _e = (call);                                                               \
        if (_e != cudaSuccess)                                                                 \
            return fail(DG_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(_e));    \
    } while (0)

double burst_pressure(const dg_params& p, double t)
{
    if (p.src_face < 0) return 0.0;
    const double T = p.src_cycles / p.src_freq;
    if (t < 0.0 || t > T) return 0.0;
    const double w = std::sin(M_PI * t / T);
    return p.src_amp * w * w * std::sin(2.0 * M_PI * p.src_freq * t + p.src_phase);
}

namespace {

// Algorithmic cost of one launch: every node's stage data moved once (values
// actually needed, neighbour faces assumed served from L2) and the FP
// operations of the formulas in dg_kernels.cuh (an FMA counts 2).
template <typename T>
double grad_bytes(const Solver& s, const StageIO<T>& io)
{
    const double nn = (double)s.gsize();
    return (1.0 + (io.inc ? 1.0 : 0.0) + 3.0) * sizeof(T) * nn;
}

double grad_flops(const Solver& s)
{
    // per axis K + 2 FMAs (line sum + two lift terms); face terms 2 flops
    const double K = s.mesh.K;
    return (3.0 * 2.0 * (K + 2.0) + 6.0 / K * 2.0) * (double)s.gsize();
}

template <typename T, bool INCR>
double stage_bytes(const Solver& s, const StageIO<T>& io)
{
    const double nn = (double)s.gsize();
    const double diff = s.p.eval_diff ? 3.0 : 0.0;
    double vals;
    if (!INCR) vals = 4.0 + diff + (io.old ? 4.0 : 0.0) + 4.0;
    else vals = 4.0 + (io.inc ? 4.0 : 0.0) + diff + 4.0 + (io.final_stage ? 8.0 : 0.0);
    return vals * sizeof(T) * nn;
}

double stage_flops(const Solver& s, bool has_old)
{
    const double K = s.mesh.K;
    const bool diff = s.p.eval_diff, adv = s.p.eval_advect;
    double f = 0.0;
    if (adv) f += 3.0 + 4.0;                              // f_mom (FMA + MUL), f_mass (ADD + 3 MUL)
    if (diff) f += 3.0;                                   // f_mass + G per axis
    f += 3.0 * 2.0 * (K + 2.0) * (adv ? 2.0 : 1.0);       // line sums + lifts (2 equations with advection)
    f += 6.0 / K * ((adv ? 21.0 : 0.0) + (diff ? 3.0 : 0.0));  // face terms (6K^2 face nodes per element)
    f += 4.0 * (2.0 + (has_old ? 2.0 : 0.0)) + 2.0;      // sponge-folded RK combination
    return f * (double)s.gsize();
}

// Per-launch operators live in a small device buffer (one slot each for the
// three RK stages, the LDG gradient and a bare right-hand side), rebuilt
// only when dt changes.
template <typename T, int K>
size_t const_slot()
{
    return (sizeof(OpConst<T, K>) + 255) / 256 * 256;
}

template <typename T, int K>
int upload_consts_k(Solver& s, double dt)
{
    const size_t slot = const_slot<T, K>();
    std::vector<char> h(5 * slot, 0);
    const double cas[5] = {dt, dt * .25, dt * 2.0 / 3.0, 0.0, 1.0};
    for (int i = 0; i < 5; i++) {
        const OpConst<T, K> C =
            i == 3 ? make_grad_const<T, K>(s.op.deriv.data(), s.op.lift0.data(), s.op.liftN.data(), s.p.elem_width,
                                           s.p.rho0, s.p.c0, s.p.diff_const)
                   : make_stage_const<T, K>(cas[i], s.op.deriv.data(), s.op.lift0.data(), s.op.liftN.data(),
                                            s.p.elem_width, s.p.rho0, s.p.c0, s.p.b_over_a, s.p.diff_const);
        std::memcpy(h.data() + i * slot, &C, sizeof C);
    }
    if (!s.d_const) {
        cudaError_t e = cudaMalloc(&s.d_const, 5 * slot);
        if (e != cudaSuccess) return fail(DG_ERR_CUDA, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    }
    // stream-ordered after every launch that used the previous operators
    cudaError_t e = cudaMemcpyAsync(s.d_const, h.data(), 5 * slot, cudaMemcpyHostToDevice, s.stream);
    if (e != cudaSuccess) return fail(DG_ERR_CUDA, std::string("cudaMemcpyAsync: ") + cudaGetErrorString(e));
    s.h_const = std::move(h);
    s.const_dt = dt;
    return DG_OK;
}

template <typename T, int K>
const OpConst<T, K>& host_const(const Solver& s, int slot)
{
    return *(const OpConst<T, K>*)(s.h_const.data() + (size_t)slot * const_slot<T, K>());
}

template <typename T, int K>
const OpConst<T, K>* const_ptr(const Solver& s, int slot)
{
    return (const OpConst<T, K>*)((const char*)s.d_const + (size_t)slot * const_slot<T, K>());
}

template <typename T, int K, bool INCR>
void launch_grad(Solver& s, const StageIO<T>& io, const MeshDev<T>& md)
{
    dim3 block(npt_of(K), epb_of(K));
    dim3 grid((md.n_elem + epb_of(K) - 1) / epb_of(K));
    cudaEvent_t ev = nullptr;
    s.prof_begin(1, &ev);
    bool done = false;
    if constexpr (!INCR && sizeof(T) == 8 && eo_grad_lines<K>()) {
        LineEO<K> L;
        if (make_line_eo<K, -1>(host_const<T, K>(s, 3), L)) {
            ldg_gradient_eo_kernel<K><<<(md.n_elem + 1) / 2, dim3(npt_of(K), 2), 0, s.stream>>>(
                io, md, const_ptr<T, K>(s, 3), L);
            done = true;
        }
    }
    if (!done)
        ldg_gradient_kernel<T, K, INCR><<<grid, block, 0, s.stream>>>(io, md, const_ptr<T, K>(s, 3),
                                                                        host_const<T, K>(s, 3));
    s.prof_end(1, ev, grad_bytes(s, io), grad_flops(s));
    s.launches++;
}

// FP64 stage kernel in the flux mode that io asks for (flux_out: write the
// output's volume fluxes; flux_in: read the input's), with even-odd line
// owners where the order has them and the operator allows them.
template <typename T, int K, bool DIFF, bool EO, int FLUX, bool PACK = false>
void launch_plain_eo(const Solver& s, const StageIO<T>& io, const MeshDev<T>& md, const OpConst<T, K>* Cp,
                     const LineEO<K>& L)
{
    const dim3 block(npt_of(K), plain_epb<K, EO>());
    const dim3 grid((md.n_elem + plain_epb<K, EO>() - 1) / plain_epb<K, EO>());
    stage_kernel<T, K, DIFF, FLUX, EO, PACK><<<grid, block, 0, s.stream>>>(io, md, Cp, L, s.p.eval_advect,
                                                                          s.p.eval_sponge);
}

// The host-order pack rides only on the flux-reading mode (the steady state
// of stepping with advection); io.pack is set only when that mode runs.
template <typename T, int K, bool DIFF, bool EO>
void launch_plain_mode(const Solver& s, const StageIO<T>& io, const MeshDev<T>& md, const OpConst<T, K>* Cp,
                       const LineEO<K>& L)
{
    if (io.flux_out && io.flux_in) {
        if (io.pack) launch_plain_eo<T, K, DIFF, EO, 2, true>(s, io, md, Cp, L);
        else launch_plain_eo<T, K, DIFF, EO, 2>(s, io, md, Cp, L);
    } else if (io.flux_out) {
        launch_plain_eo<T, K, DIFF, EO, 1>(s, io, md, Cp, L);
    } else {
        launch_plain_eo<T, K, DIFF, EO, 0>(s, io, md, Cp, L);
    }
}

template <typename T, int K, bool DIFF>
void launch_plain(const Solver& s, int slot, const StageIO<T>& io, const MeshDev<T>& md, const OpConst<T, K>* Cp)
{
    LineEO<K> L{};
    if constexpr (sizeof(T) == 8 && eo_lines<K>()) {
        if (make_line_eo<K, 1>(host_const<T, K>(s, slot), L)) {
            launch_plain_mode<T, K, DIFF, true>(s, io, md, Cp, L);
            return;
        }
    }
    launch_plain_mode<T, K, DIFF, false>(s, io, md, Cp, L);
}

template <typename T, int K, bool INCR>
void launch_stage(Solver& s, const StageIO<T>& io, const MeshDev<T>& md, int slot)
{
    const OpConst<T, K>* Cp = const_ptr<T, K>(s, slot);
    cudaEvent_t ev = nullptr;
    s.prof_begin(0, &ev);
    if constexpr (INCR) {
        const dim3 block(npt_of(K), epb_of(K));
        const dim3 grid((md.n_elem + epb_of(K) - 1) / epb_of(K));
        const OpConst<T, K>& Cv = host_const<T, K>(s, slot);
        if (s.p.eval_diff)
            incr_stage_kernel<T, K, true><<<grid, block, 0, s.stream>>>(io, md, Cp, Cv, s.p.eval_advect,
                                                                       s.p.eval_sponge);
        else
            incr_stage_kernel<T, K, false><<<grid, block, 0, s.stream>>>(io, md, Cp, Cv, s.p.eval_advect,
                                                                        s.p.eval_sponge);
    } else {
        if (s.p.eval_diff) launch_plain<T, K, true>(s, slot, io, md, Cp);
        else launch_plain<T, K, false>(s, slot, io, md, Cp);
    }
    s.prof_end(0, ev, stage_bytes<T, INCR>(s, io), stage_flops(s, io.old != nullptr || io.inc != nullptr));
    s.launches++;
}

// FP64 plain form: the stage input's weight with the sponge folded in,
// cb - ca sigma_e, per element for each of the three RK stages (stage-major),
// so that the stage kernel reads it instead of computing it at every node.
int upload_elem_weights(Solver& s, double dt)
{
    const size_t ne = (size_t)s.mesh.n_elem;
    const double w23 = s.p.rk_exact ? 2.0 / 3.0 : (double)(2.0f / 3.0f);
    const double ca[3] = {dt, dt * .25, dt * 2.0 / 3.0}, cb[3] = {1.0, .25, w23};
    std::vector<double>& h = s.h_elem_b;
    h.resize(3 * ne);
    for (int k = 0; k < 3; k++)
        for (size_t e = 0; e < ne; e++) h[k * ne + e] = s.p.eval_sponge ? cb[k] - ca[k] * s.mesh.sigma[e] : cb[k];
    if (!s.d_elem_b) {
        cudaError_t e = cudaMalloc(&s.d_elem_b, h.size() * sizeof(double));
        if (e != cudaSuccess) return fail(DG_ERR_CUDA, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    }
    cudaError_t e = cudaMemcpyAsync(s.d_elem_b, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice, s.stream);
    if (e != cudaSuccess) return fail(DG_ERR_CUDA, std::string("cudaMemcpyAsync: ") + cudaGetErrorString(e));
    return DG_OK;
}

template <typename T>
int upload_consts(Solver& s, double dt)
{
    if constexpr (sizeof(T) == 8) {
        int rc = upload_elem_weights(s, dt);
        if (rc) return rc;
    }
    switch (s.mesh.K) {
    case 2: return upload_consts_k<T, 2>(s, dt);
    case 3: return upload_consts_k<T, 3>(s, dt);
    case 4: return upload_consts_k<T, 4>(s, dt);
    case 5: return upload_consts_k<T, 5>(s, dt);
    case 6: return upload_consts_k<T, 6>(s, dt);
    case 7: return upload_consts_k<T, 7>(s, dt);
    case 8: return upload_consts_k<T, 8>(s, dt);
    }
    return fail(DG_ERR_INVALID, "unsupported order");
}

template <typename T, bool INCR>
void dispatch_grad(Solver& s, const StageIO<T>& io, const MeshDev<T>& md)
{
    switch (s.mesh.K) {
    case 2: launch_grad<T, 2, INCR>(s, io, md); break;
    case 3: launch_grad<T, 3, INCR>(s, io, md); break;
    case 4: launch_grad<T, 4, INCR>(s, io, md); break;
    case 5: launch_grad<T, 5, INCR>(s, io, md); break;
    case 6: launch_grad<T, 6, INCR>(s, io, md); break;
    case 7: launch_grad<T, 7, INCR>(s, io, md); break;
    case 8: launch_grad<T, 8, INCR>(s, io, md); break;
    }
}

template <typename T, bool INCR>
void dispatch_stage(Solver& s, const StageIO<T>& io, const MeshDev<T>& md, int slot)
{
    switch (s.mesh.K) {
    case 2: launch_stage<T, 2, INCR>(s, io, md, slot); break;
    case 3: launch_stage<T, 3, INCR>(s, io, md, slot); break;
    case 4: launch_stage<T, 4, INCR>(s, io, md, slot); break;
    case 5: launch_stage<T, 5, INCR>(s, io, md, slot); break;
    case 6: launch_stage<T, 6, INCR>(s, io, md, slot); break;
    case 7: launch_stage<T, 7, INCR>(s, io, md, slot); break;
    case 8: launch_stage<T, 8, INCR>(s, io, md, slot); break;
    }
}

template <typename T>
MeshDev<T> mesh_dev(const Solver& s)
{
    MeshDev<T> m;
    m.nbr = s.d_nbr;
    m.sigma = (const T*)s.d_sigma;
    m.bnd_ic = (const T*)s.d_bnd_ic;
    m.bnd_ap = (const T*)s.d_bnd_ap;
    m.bnd_src = s.d_bnd_src;
    m.n_elem = s.mesh.n_elem;
    m.ic_live = 0;
    m.src_p = T(0);
    return m;
}

template <typename T>
int upload_as(const std::vector<double>& h, void** d)
{
    std::vector<T> tmp(h.begin(), h.end());
    size_t bytes = std::max<size_t>(tmp.size(), 1) * sizeof(T);
    DG_CUDA(cudaMalloc(d, bytes));
    if (!tmp.empty()) DG_CUDA(cudaMemcpy(*d, tmp.data(), tmp.size() * sizeof(T), cudaMemcpyHostToDevice));
    return DG_OK;
}

GridMap grid_map(const MeshHost& m)
{
    GridMap g;
    g.K = m.K;
    for (int a = 0; a < 3; a++) {
        g.nb[a] = m.nb[a];
        g.ne[a] = m.ne[a];
        g.E[a] = m.E[a];
    }
    g.elem_per_block = m.elem_per_block;
    return g;
}

}  // namespace

// ---------------------------------------------------------------------------
// One RK step (three stages) in each precision.
// ---------------------------------------------------------------------------
int Solver::rk_stage_fp64(int s_idx, double dt, double* rhs_only)
{
    MeshDev<double> md = mesh_dev<double>(*this);
    const double w23 = p.rk_exact ? 2.0 / 3.0 : (double)(2.0f / 3.0f);
    const double w13 = p.rk_exact ? 1.0 / 3.0 : (double)(1.0f / 3.0f);
    const double tst[3] = {t, t + dt, t + 0.5 * dt};
    double* U = (double*)buf[0];
    double* k1 = (double*)buf[1];
    double* k2 = (double*)buf[2];
    StageIO<double> io;
    std::memset(&io, 0, sizeof io);
    io.fs = mesh.fstride();
    io.np = mesh.NP;
    io.q = (const double*)qbuf;
    io.q_out = (double*)qbuf;
    if (rhs_only) {
        io.src = U;
        io.dst = rhs_only;
        io.ca = 1.0;
        io.cb = 0.0;
    } else if (s_idx == 0) {
        io.src = U; io.dst = k1; io.old = nullptr; io.ca = dt; io.cb = 1.0; io.cc = 0.0;
    } else if (s_idx == 1) {
        io.src = k1; io.dst = k2; io.old = U; io.ca = dt * .25; io.cb = .25; io.cc = .75;
    } else {
        io.src = k2; io.dst = U; io.old = U; io.ca = dt * 2.0 / 3.0; io.cb = w23; io.cc = w13;
    }
    md.ic_live = (s_idx == 0 && ic_live) ? 1 : 0;
    md.src_p = burst_pressure(p, tst[s_idx]);
    if (!d_const || (!rhs_only && dt != const_dt)) {
        int rc = upload_consts<double>(*this, dt);
        if (rc) return rc;
    }
    const bool fluxes = !rhs_only && d_flux[0];
    if (!rhs_only) io.elem_b = d_elem_b + (size_t)s_idx * mesh.n_elem;
    if (fluxes) {
        io.flux_in = flux_valid ? d_flux[flux_cur] : nullptr;
        io.flux_out = d_flux[1 - flux_cur];
    }
    if (s_idx == 2 && !rhs_only && stage3_pack && io.flux_in && io.flux_out) {
        io.pack = stage3_pack;
        io.pack_map = grid_map(mesh);
        io.pack_gsize = gsize();
        stage3_packed = true;
    }
    if (p.eval_diff) dispatch_grad<double, false>(*this, io, md);
    dispatch_stage<double, false>(*this, io, md, rhs_only ? 4 : s_idx);
    if (fluxes) {
        flux_cur = 1 - flux_cur;
        flux_valid = true;
    }
    return DG_OK;
}

int Solver::rk_stage_fp32(int s_idx, double dt, float* rhs_only)
{
    MeshDev<float> md = mesh_dev<float>(*this);
    const double w23 = p.rk_exact ? 2.0 / 3.0 : (double)(2.0f / 3.0f);
    const double w13 = p.rk_exact ? 1.0 / 3.0 : (double)(1.0f / 3.0f);
    const double tst[3] = {t, t + dt, t + 0.5 * dt};
    float* u = (float*)buf[cur];
    float* unext = (float*)buf[1 - cur];
    float* comp = (float*)buf[2];
    float* d1 = (float*)buf[3];
    float* d2 = (float*)buf[4];
    const double cas[3] = {dt, dt * .25, dt * 2.0 / 3.0};
    const double ca = rhs_only ? 1.0 : cas[s_idx];
    StageIO<float> io;
    std::memset(&io, 0, sizeof io);
    io.fs = mesh.fstride();
    io.np = mesh.NP;
    io.q = (const float*)qbuf;
    io.q_out = (float*)qbuf;
    io.src = u;
    if (rhs_only) {
        io.dst = rhs_only;
        io.ca = 1.0f;
    } else if (s_idx == 0) {
        io.dst = d1;
        io.ca = (float)dt;
    } else if (s_idx == 1) {
        io.inc = d1; io.dst = d2; io.ca = (float)(dt * .25); io.cb = .25f;
    } else {
        io.inc = d2; io.dst = unext; io.comp = comp; io.final_stage = 1;
        io.ca = (float)(dt * 2.0 / 3.0);
        io.cb = (float)w23;
        io.eps = (float)(w23 + w13 - 1.0);
    }
    md.ic_live = (s_idx == 0 && ic_live) ? 1 : 0;
    md.src_p = (float)burst_pressure(p, tst[s_idx]);
    if (!d_const || (!rhs_only && dt != const_dt)) {
        int rc = upload_consts<float>(*this, dt);
        if (rc) return rc;
    }
    (void)ca;
    if (p.eval_diff) dispatch_grad<float, true>(*this, io, md);
    dispatch_stage<float, true>(*this, io, md, rhs_only ? 4 : s_idx);
    return DG_OK;
}

template <typename T>
__global__ void probe_kernel(const T* __restrict__ state, size_t fs, const long long* __restrict__ off, int n,
                             double* __restrict__ row, double c2, double kba)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double d = (double)state[off[i]];
    row[i] = c2 * (d + kba * d * d);
    (void)fs;
}

int Solver::probe_reserve(long long steps)
{
    if (n_probe == 0 || steps <= probe_cap) return DG_OK;
    long long cap = std::max<long long>(steps, 2 * probe_cap + 64);
    double* nb = nullptr;
    DG_CUDA(cudaMalloc(&nb, (size_t)cap * n_probe * sizeof(double)));
    if (d_probe_rec && probe_steps)
        DG_CUDA(cudaMemcpyAsync(nb, d_probe_rec, (size_t)probe_steps * n_probe * sizeof(double),
                                cudaMemcpyDeviceToDevice, stream));
    DG_CUDA(cudaStreamSynchronize(stream));
    if (d_probe_rec) cudaFree(d_probe_rec);
    d_probe_rec = nb;
    probe_cap = cap;
    return DG_OK;
}

void Solver::probe_record()
{
    if (n_probe == 0) return;
    const double c2 = p.c0 * p.c0, kba = p.b_over_a / (2.0 * p.rho0);
    double* row = d_probe_rec + (size_t)probe_steps * n_probe;
    if (fp64())
        probe_kernel<double><<<(n_probe + 127) / 128, 128, 0, stream>>>((const double*)state_ptr(), mesh.fstride(),
                                                                       d_probe_off, n_probe, row, c2, kba);
    else
        probe_kernel<float><<<(n_probe + 127) / 128, 128, 0, stream>>>((const float*)state_ptr(), mesh.fstride(),
                                                                      d_probe_off, n_probe, row, c2, kba);
    launches++;
    probe_t.push_back(t);
    probe_steps++;
}

int Solver::step(double dt, int nsteps)
{
    if (n_probe) {
        int rc = probe_reserve(probe_steps + nsteps);
        if (rc) return rc;
    }
    for (int n = 0; n < nsteps; n++) {
        for (int s = 0; s < 3; s++) {
            // stage 3 writes U in place (FP64) or the other u buffer (FP32)
            if (s == 2) wait_pack(stream, fp64() ? buf[0] : buf[1 - cur]);
            int rc = fp64() ? rk_stage_fp64(s, dt, nullptr) : rk_stage_fp32(s, dt, nullptr);
            if (rc) return rc;
        }
        DG_CUDA(cudaGetLastError());
        if (!fp64()) cur = 1 - cur;
        ic_live = false;
        t += dt;
        steps_done++;
        probe_record();
    }
    return DG_OK;
}

int Solver::eval_rhs(double* drho, double* vel)
{
    // R = L(current state) into the k1 / d1 buffer, then pack.
    if (fp64()) rk_stage_fp64(0, 0.0, (double*)buf[1]);
    else rk_stage_fp32(0, 0.0, (float*)buf[3]);
    DG_CUDA(cudaGetLastError());
    return pack_out(fp64() ? buf[1] : buf[3], drho, vel);
}

void* Solver::state_ptr() const { return fp64() ? buf[0] : buf[cur]; }

int Solver::ensure_staging()
{
    if (staging) return DG_OK;
    DG_CUDA(cudaMalloc(&staging, 4 * gsize() * sizeof(double)));
    return DG_OK;
}

namespace {

// Device address of pinned (page-locked, mapped) host memory, or null when the
// pointer is ordinary pageable memory that a kernel must not touch.
const void* device_view(const void* host)
{
    if (!host) return nullptr;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, host) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return (a.type == cudaMemoryTypeHost && a.devicePointer) ? a.devicePointer : nullptr;
}

}  // namespace

// Host transfers.  Pinned host buffers are read/written directly by the
// host-order kernels over the CPU-GPU link (no staging copy); pageable ones go
// through the device staging buffer and bulk copies.
int Solver::pack_out(const void* src, double* drho, double* vel)
{
    const GridMap g = grid_map(mesh);
    const int threads = 128, blocks = 152 * 16;
    double* rho_d = (double*)device_view(drho);
    double* vel_d = (double*)device_view(vel);
    const bool direct = (!drho || rho_d) && (!vel || vel_d);
    if (!direct) {
        int rc = ensure_staging();
        if (rc) return rc;
        rho_d = drho ? staging : nullptr;
        vel_d = vel ? staging + gsize() : nullptr;
    }
    if (fp64())
        pack_host_order_kernel<double><<<blocks, threads, 0, stream>>>((const double*)src, mesh.fstride(), mesh.NP, g,
                                                                       rho_d, vel_d, gsize());
    else
        pack_host_order_kernel<float><<<blocks, threads, 0, stream>>>((const float*)src, mesh.fstride(), mesh.NP, g,
                                                                      rho_d, vel_d, gsize());
    launches++;
    DG_CUDA(cudaGetLastError());
    if (!direct) {
        if (drho) DG_CUDA(cudaMemcpyAsync(drho, staging, gsize() * sizeof(double), cudaMemcpyDeviceToHost, stream));
        if (vel)
            DG_CUDA(cudaMemcpyAsync(vel, staging + gsize(), 3 * gsize() * sizeof(double), cudaMemcpyDeviceToHost,
                                    stream));
    }
    DG_CUDA(cudaStreamSynchronize(stream));
    return DG_OK;
}

int Solver::unpack_in(const double* drho, const double* vel)
{
    wait_pack(stream, state_ptr());
    const double* rho_d = (const double*)device_view(drho);
    const double* vel_d = (const double*)device_view(vel);
    const bool staged = !rho_d || !vel_d;
    if (staged) {
        int rc = ensure_staging();
        if (rc) return rc;
        DG_CUDA(cudaMemcpyAsync(staging, drho, gsize() * sizeof(double), cudaMemcpyHostToDevice, stream));
        DG_CUDA(cudaMemcpyAsync(staging + gsize(), vel, 3 * gsize() * sizeof(double), cudaMemcpyHostToDevice, stream));
        rho_d = staging;
        vel_d = staging + gsize();
    }
    int rc = launch_unpack(rho_d, vel_d, staged);
    if (rc) return rc;
    DG_CUDA(cudaStreamSynchronize(stream));
    return DG_OK;
}

// Host-order device staging -> state on stream st, walked in element order.
template <typename T>
cudaError_t Solver::launch_unpack_staged(T* state, const GridMap& g, const double* rho_d, const double* vel_d,
                                         const FluxOut<T>& fo, cudaStream_t st)
{
    unpack_elem_order_kernel<T><<<152 * 16, 256, 0, st>>>(state, mesh.fstride(), mesh.NP, g, mesh.n_elem, rho_d,
                                                          vel_d, gsize(), fo);
    return cudaGetLastError();
}

// Host-order arrays -> state on the compute stream: device staging walked in
// element order, pinned host memory (read over the CPU-GPU link) in host
// order.
int Solver::launch_unpack(const double* rho_d, const double* vel_d, bool on_device)
{
    const GridMap g = grid_map(mesh);
    const int threads = 128, blocks = 152 * 16;
    // FP64 with advection: the unpack also writes the state's volume fluxes
    // for the next stage to read.
    const FluxOut<double> fo = flux_consts<double>(d_flux[flux_cur], p.rho0, p.c0, p.b_over_a);
    const FluxOut<float> none = flux_consts<float>(nullptr, p.rho0, p.c0, p.b_over_a);
    if (on_device) {
        cudaError_t e = fp64() ? launch_unpack_staged<double>((double*)state_ptr(), g, rho_d, vel_d, fo, stream)
                               : launch_unpack_staged<float>((float*)state_ptr(), g, rho_d, vel_d, none, stream);
        if (e != cudaSuccess) return fail(DG_ERR_CUDA, std::string("unpack: ") + cudaGetErrorString(e));
    } else {
        if (fp64())
            unpack_host_order_kernel<double><<<blocks, threads, 0, stream>>>((double*)state_ptr(), mesh.fstride(),
                                                                             mesh.NP, g, rho_d, vel_d, gsize(), fo);
        else
            unpack_host_order_kernel<float><<<blocks, threads, 0, stream>>>((float*)state_ptr(), mesh.fstride(),
                                                                            mesh.NP, g, rho_d, vel_d, gsize(), none);
    }
    launches++;
    DG_CUDA(cudaGetLastError());
    if (!fp64()) DG_CUDA(cudaMemsetAsync(buf[2], 0, 4 * mesh.fstride() * sizeof(float), stream));  // Kahan compensation
    flux_valid = fp64() && d_flux[0] != nullptr;
    ic_live = false;
    return DG_OK;
}

void Solver::wait_pack(cudaStream_t st, const void* target)
{
    for (const PackEvent& pe : pack_ev)
        if (pe.ev && pe.src == target) cudaStreamWaitEvent(st, pe.ev, 0);
}

int Solver::ensure_async()
{
    // Each resource is created once; a call after a failed one resumes here.
    if (!copy_in) DG_CUDA(cudaStreamCreateWithFlags(&copy_in, cudaStreamNonBlocking));
    if (!copy_out) DG_CUDA(cudaStreamCreateWithFlags(&copy_out, cudaStreamNonBlocking));
    // the transposes share the SMs with the steps at the compute stream's
    // priority (a higher one measured slightly slower end to end)
    if (!xin) DG_CUDA(cudaStreamCreateWithFlags(&xin, cudaStreamNonBlocking));
    if (!xout) DG_CUDA(cudaStreamCreateWithFlags(&xout, cudaStreamNonBlocking));
    const size_t es = fp64() ? sizeof(double) : sizeof(float);
    if (!spare_u) DG_CUDA(cudaMalloc(&spare_u, 4 * mesh.fstride() * es));
    if (fp64() && d_flux[0] && !spare_f) DG_CUDA(cudaMalloc(&spare_f, 4 * mesh.fstride() * sizeof(double)));
    for (cudaEvent_t* e : {&spare_ready, &spare_free, &step_done})
        if (!*e) DG_CUDA(cudaEventCreateWithFlags(e, cudaEventDisableTiming));
    for (PackEvent& pe : pack_ev)
        if (!pe.ev) DG_CUDA(cudaEventCreateWithFlags(&pe.ev, cudaEventDisableTiming));
    for (int i = 0; i < 2; i++) {
        if (!astage_in[i]) DG_CUDA(cudaMalloc(&astage_in[i], 4 * gsize() * sizeof(double)));
        if (!astage_out[i]) DG_CUDA(cudaMalloc(&astage_out[i], 4 * gsize() * sizeof(double)));
        for (cudaEvent_t* e : {&in_ready[i], &in_free[i], &out_ready[i], &out_free[i]})
            if (!*e) DG_CUDA(cudaEventCreateWithFlags(e, cudaEventDisableTiming));
    }
    return DG_OK;
}

// Upload on the copy-in stream into staging slot k; unpack on the xin stream
// into the spare state (and flux) buffer once the steps and the pack that
// last used it are done, so it runs under the step enqueued before; the
// compute stream swaps it in at this point of the call sequence.  The slot is
// reused only after the unpack that last read it.
int Solver::set_state_async(const double* drho, const double* vel)
{
    if (!device_view(drho) || !device_view(vel))
        return fail(DG_ERR_INVALID, "dg_set_state_async: host buffers must be page-locked (pinned)");
    int rc = ensure_async();
    if (rc) return rc;
    const int k = in_slot;
    in_slot ^= 1;
    const size_t n = gsize();
    double* st = astage_in[k];
    DG_CUDA(cudaStreamWaitEvent(copy_in, in_free[k], 0));
    DG_CUDA(cudaMemcpyAsync(st, drho, n * sizeof(double), cudaMemcpyHostToDevice, copy_in));
    DG_CUDA(cudaMemcpyAsync(st + n, vel, 3 * n * sizeof(double), cudaMemcpyHostToDevice, copy_in));
    DG_CUDA(cudaEventRecord(in_ready[k], copy_in));
    DG_CUDA(cudaStreamWaitEvent(xin, in_ready[k], 0));
    if (spare_free_recorded) DG_CUDA(cudaStreamWaitEvent(xin, spare_free, 0));
    wait_pack(xin, spare_u);
    const GridMap g = grid_map(mesh);
    cudaError_t e;
    if (fp64()) {
        const FluxOut<double> fo = flux_consts<double>(spare_f, p.rho0, p.c0, p.b_over_a);
        e = launch_unpack_staged<double>((double*)spare_u, g, st, st + n, fo, xin);
    } else {
        const FluxOut<float> none = flux_consts<float>(nullptr, p.rho0, p.c0, p.b_over_a);
        e = launch_unpack_staged<float>((float*)spare_u, g, st, st + n, none, xin);
    }
    if (e != cudaSuccess) return fail(DG_ERR_CUDA, std::string("unpack: ") + cudaGetErrorString(e));
    launches++;
    DG_CUDA(cudaEventRecord(in_free[k], xin));
    DG_CUDA(cudaEventRecord(spare_ready, xin));
    // swap the uploaded state (and its fluxes) in on the compute stream
    DG_CUDA(cudaStreamWaitEvent(stream, spare_ready, 0));
    void*& cur_u = fp64() ? buf[0] : buf[cur];
    std::swap(cur_u, spare_u);
    if (spare_f) std::swap(d_flux[flux_cur], spare_f);
    if (!fp64()) DG_CUDA(cudaMemsetAsync(buf[2], 0, 4 * mesh.fstride() * sizeof(float), stream));  // Kahan compensation
    flux_valid = fp64() && d_flux[0] != nullptr;
    ic_live = false;
    // the buffers swapped out are free once the work enqueued so far is done
    DG_CUDA(cudaEventRecord(spare_free, stream));
    spare_free_recorded = true;
    return DG_OK;
}

// Pack on the xout stream into staging slot k (after the steps enqueued so
// far and the download that last read the slot), then download on the
// copy-out stream.  The compute stream goes on with the next steps and waits
// for this pack only before it writes the state buffer the pack reads.
int Solver::get_state_async(double* drho, double* vel)
{
    if ((drho && !device_view(drho)) || (vel && !device_view(vel)))
        return fail(DG_ERR_INVALID, "dg_get_state_async: host buffers must be page-locked (pinned)");
    int rc = ensure_async();
    if (rc) return rc;
    const int k = out_slot;
    out_slot ^= 1;
    const size_t n = gsize();
    double* st = astage_out[k];
    DG_CUDA(cudaEventRecord(step_done, stream));
    DG_CUDA(cudaStreamWaitEvent(xout, step_done, 0));
    DG_CUDA(cudaStreamWaitEvent(xout, out_free[k], 0));
    const GridMap g = grid_map(mesh);
    const int threads = 128, blocks = 152 * 16;
    if (fp64())
        pack_host_order_kernel<double><<<blocks, threads, 0, xout>>>((const double*)state_ptr(), mesh.fstride(),
                                                                     mesh.NP, g, drho ? st : nullptr,
                                                                     vel ? st + n : nullptr, n);
    else
        pack_host_order_kernel<float><<<blocks, threads, 0, xout>>>((const float*)state_ptr(), mesh.fstride(),
                                                                    mesh.NP, g, drho ? st : nullptr,
                                                                    vel ? st + n : nullptr, n);
    launches++;
    DG_CUDA(cudaGetLastError());
    DG_CUDA(cudaEventRecord(out_ready[k], xout));
    // one event per state buffer: the pack of this buffer is done
    PackEvent* pe = nullptr;
    for (PackEvent& x : pack_ev)
        if (x.src == state_ptr()) pe = &x;
    for (PackEvent& x : pack_ev)
        if (!pe && !x.src) pe = &x;
    if (!pe) return fail(DG_ERR_STATE, "dg_get_state_async: more state buffers than pack events");
    pe->src = state_ptr();
    DG_CUDA(cudaEventRecord(pe->ev, xout));
    DG_CUDA(cudaStreamWaitEvent(copy_out, out_ready[k], 0));
    if (drho) DG_CUDA(cudaMemcpyAsync(drho, st, n * sizeof(double), cudaMemcpyDeviceToHost, copy_out));
    if (vel) DG_CUDA(cudaMemcpyAsync(vel, st + n, 3 * n * sizeof(double), cudaMemcpyDeviceToHost, copy_out));
    DG_CUDA(cudaEventRecord(out_free[k], copy_out));
    return DG_OK;
}

// One step whose result is downloaded: in the FP64 path with advection the
// last stage writes its output in host order into staging slot k as well (no
// pack kernel), then the download runs on the copy-out stream; otherwise a
// step and dg_get_state_async.
int Solver::step_get_async(double dt, double* drho, double* vel)
{
    if (!device_view(drho) || !device_view(vel))
        return fail(DG_ERR_INVALID, "dg_step_get_state_async: host buffers must be page-locked (pinned)");
    int rc = ensure_async();
    if (rc) return rc;
    if (!(fp64() && d_flux[0])) {
        rc = step(dt, 1);
        return rc ? rc : get_state_async(drho, vel);
    }
    const int k = out_slot;
    out_slot ^= 1;
    const size_t n = gsize();
    double* st = astage_out[k];
    DG_CUDA(cudaStreamWaitEvent(stream, out_free[k], 0));  // the download that last read the slot
    stage3_pack = st;
    stage3_packed = false;
    rc = step(dt, 1);
    stage3_pack = nullptr;
    if (rc) return rc;
    if (!stage3_packed) {
        // the last stage ran in a mode without the pack: pack separately
        const GridMap g = grid_map(mesh);
        pack_host_order_kernel<double><<<152 * 16, 128, 0, stream>>>((const double*)state_ptr(), mesh.fstride(),
                                                                     mesh.NP, g, st, st + n, n);
        launches++;
        DG_CUDA(cudaGetLastError());
    }
    DG_CUDA(cudaEventRecord(out_ready[k], stream));
    DG_CUDA(cudaStreamWaitEvent(copy_out, out_ready[k], 0));
    DG_CUDA(cudaMemcpyAsync(drho, st, n * sizeof(double), cudaMemcpyDeviceToHost, copy_out));
    DG_CUDA(cudaMemcpyAsync(vel, st + n, 3 * n * sizeof(double), cudaMemcpyDeviceToHost, copy_out));
    DG_CUDA(cudaEventRecord(out_free[k], copy_out));
    return DG_OK;
}

int Solver::sync_all()
{
    DG_CUDA(cudaStreamSynchronize(stream));
    if (xin) DG_CUDA(cudaStreamSynchronize(xin));
    if (xout) DG_CUDA(cudaStreamSynchronize(xout));
    if (copy_in) DG_CUDA(cudaStreamSynchronize(copy_in));
    if (copy_out) DG_CUDA(cudaStreamSynchronize(copy_out));
    return DG_OK;
}

size_t Solver::device_bytes() const
{
    const size_t fs = mesh.fstride();
    const size_t es = fp64() ? 8 : 4;
    size_t nbuf = fp64() ? 3 : 5;  // FP64: U, k1, k2; FP32: u0, u1, comp, d1, d2
    size_t bytes = nbuf * 4 * fs * es + 3 * fs * es;
    if (fp64() && p.eval_advect) bytes += 2 * 4 * fs * es;  // volume-flux buffers
    bytes += (size_t)mesh.n_elem * 6 * sizeof(int) + (size_t)mesh.n_elem * es;
    bytes += (size_t)mesh.n_bnd * (3 * mesh.K * mesh.K * es + sizeof(int));
    return bytes;
}

int Solver::init(const dg_params& prm, const char* matrix_file, const char* coeff_file)
{
    p = prm;
    std::string err = validate_params(p);
    if (!err.empty()) return fail(DG_ERR_INVALID, err);
    err = build_line_operators(p.order, p.lumped_mass != 0, matrix_file ? matrix_file : "",
                               coeff_file ? coeff_file : "", op);
    if (!err.empty()) return fail(err.find("Opening") == 0 ? DG_ERR_IO : DG_ERR_INVALID, err);
    err = build_mesh(p, op, mesh);
    if (!err.empty()) return fail(DG_ERR_INVALID, err);

    DG_CUDA(cudaGetDevice(&device));
    size_t free_b = 0, total_b = 0;
    DG_CUDA(cudaMemGetInfo(&free_b, &total_b));
    const size_t need = device_bytes();
    if (need > free_b)
        return fail(DG_ERR_NOMEM, "state needs " + std::to_string(need) + " bytes, device has " +
                                      std::to_string(free_b) + " free");
    DG_CUDA(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));

    const size_t fs = mesh.fstride();
    const size_t es = fp64() ? 8 : 4;
    const int nbuf = fp64() ? 3 : 5;
    for (int i = 0; i < nbuf; i++) {
        DG_CUDA(cudaMalloc(&buf[i], 4 * fs * es));
        DG_CUDA(cudaMemsetAsync(buf[i], 0, 4 * fs * es, stream));
    }
    DG_CUDA(cudaMalloc(&qbuf, 3 * fs * es));
    if (fp64() && p.eval_advect)
        for (double*& f : d_flux) DG_CUDA(cudaMalloc(&f, 4 * fs * es));
    flux_valid = false;
    DG_CUDA(cudaMemsetAsync(qbuf, 0, 3 * fs * es, stream));
    DG_CUDA(cudaMalloc(&d_nbr, mesh.nbr.size() * sizeof(int)));
    DG_CUDA(cudaMemcpy(d_nbr, mesh.nbr.data(), mesh.nbr.size() * sizeof(int), cudaMemcpyHostToDevice));
    std::vector<int> is_src(std::max(mesh.n_bnd, 1), 0);
    for (int b = 0; b < mesh.n_bnd; b++) is_src[b] = mesh.bnd_face[b] == p.src_face ? 1 : 0;
    DG_CUDA(cudaMalloc(&d_bnd_src, is_src.size() * sizeof(int)));
    DG_CUDA(cudaMemcpy(d_bnd_src, is_src.data(), is_src.size() * sizeof(int), cudaMemcpyHostToDevice));
    int rc;
    if (fp64()) {
        if ((rc = upload_as<double>(mesh.sigma, &d_sigma))) return rc;
        if ((rc = upload_as<double>(mesh.bnd_ic, &d_bnd_ic))) return rc;
        if ((rc = upload_as<double>(mesh.bnd_ap, &d_bnd_ap))) return rc;
        DG_CUDA(cudaMemcpy(buf[0], mesh.state0.data(), 4 * fs * sizeof(double), cudaMemcpyHostToDevice));
    } else {
        if ((rc = upload_as<float>(mesh.sigma, &d_sigma))) return rc;
        if ((rc = upload_as<float>(mesh.bnd_ic, &d_bnd_ic))) return rc;
        if ((rc = upload_as<float>(mesh.bnd_ap, &d_bnd_ap))) return rc;
        std::vector<float> s0(mesh.state0.begin(), mesh.state0.end());
        DG_CUDA(cudaMemcpy(buf[0], s0.data(), 4 * fs * sizeof(float), cudaMemcpyHostToDevice));
        cur = 0;
    }
    DG_CUDA(cudaStreamSynchronize(stream));
    // The initial state lives on the device now; keep no host copy of it.
    std::vector<double>().swap(mesh.state0);
    ic_live = true;
    t = 0.0;
    return DG_OK;
}

cudaEvent_t Solver::take_event()
{
    if (!event_pool.empty()) {
        cudaEvent_t e = event_pool.back();
        event_pool.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
    return e;
}

void Solver::prof_begin(int k, cudaEvent_t* a)
{
    (void)k;
    *a = nullptr;
    if (!profiling) return;
    *a = take_event();
    if (*a) cudaEventRecord(*a, stream);
}

void Solver::prof_end(int k, cudaEvent_t a, double bytes, double flops)
{
    if (!profiling) return;
    KernelStat& st = kstat[k];
    st.launches++;
    st.bytes += bytes;
    st.flops += flops;
    if (!a) return;
    cudaEvent_t b = take_event();
    if (!b) return;
    cudaEventRecord(b, stream);
    st.ev.emplace_back(a, b);
}

void Solver::prof_reset()
{
    for (KernelStat& st : kstat) {
        for (auto& pr : st.ev) {
            event_pool.push_back(pr.first);
            event_pool.push_back(pr.second);
        }
        st.ev.clear();
        st.launches = 0;
        st.bytes = st.flops = 0.0;
    }
}

Solver::~Solver()
{
    if (stream) cudaStreamSynchronize(stream);
    for (cudaStream_t c : {xin, xout, copy_in, copy_out})
        if (c) {
            cudaStreamSynchronize(c);
            cudaStreamDestroy(c);
        }
    for (int i = 0; i < 2; i++) {
        for (double* b : {astage_in[i], astage_out[i]})
            if (b) cudaFree(b);
        for (cudaEvent_t e : {in_ready[i], in_free[i], out_ready[i], out_free[i]})
            if (e) cudaEventDestroy(e);
    }
    for (cudaEvent_t e : {spare_ready, spare_free, step_done})
        if (e) cudaEventDestroy(e);
    for (PackEvent& pe : pack_ev)
        if (pe.ev) cudaEventDestroy(pe.ev);
    if (spare_u) cudaFree(spare_u);
    if (spare_f) cudaFree(spare_f);
    prof_reset();
    for (cudaEvent_t e : event_pool) cudaEventDestroy(e);
    for (void* b : buf)
        if (b) cudaFree(b);
    if (qbuf) cudaFree(qbuf);
    if (staging) cudaFree(staging);
    if (d_nbr) cudaFree(d_nbr);
    if (d_sigma) cudaFree(d_sigma);
    if (d_bnd_ic) cudaFree(d_bnd_ic);
    if (d_bnd_ap) cudaFree(d_bnd_ap);
    if (d_bnd_src) cudaFree(d_bnd_src);
    if (d_const) cudaFree(d_const);
    if (d_elem_b) cudaFree(d_elem_b);
    for (double* f : d_flux)
        if (f) cudaFree(f);
    if (d_probe_off) cudaFree(d_probe_off);
    if (d_probe_rec) cudaFree(d_probe_rec);
    if (stream) cudaStreamDestroy(stream);
}

}  // namespace dg

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
using dg::fail;
using dg::Solver;

extern "C" {

int dg_create(const dg_params* p, const char* matrix_file, const char* coeff_file, dg_handle** out)
{
    if (!p || !out) return fail(DG_ERR_INVALID, "dg_create: null argument");
    *out = nullptr;
    dg_handle* h = new (std::nothrow) dg_handle;
    if (!h) return fail(DG_ERR_NOMEM, "dg_create: host allocation failed");
    int rc = h->s.init(*p, matrix_file, coeff_file);
    if (rc) {
        delete h;
        return rc;
    }
    dg::g_last_error.clear();
    *out = h;
    return DG_OK;
}

int dg_destroy(dg_handle* h)
{
    delete h;
    return DG_OK;
}

int dg_step(dg_handle* h, double dt, int nsteps)
{
    if (!h) return fail(DG_ERR_INVALID, "dg_step: null handle");
    if (nsteps < 0 || !std::isfinite(dt)) return fail(DG_ERR_INVALID, "dg_step: bad dt or nsteps");
    return h->s.step(dt, nsteps);
}

int dg_synchronize(dg_handle* h)
{
    if (!h) return fail(DG_ERR_INVALID, "dg_synchronize: null handle");
    return h->s.sync_all();
}

int dg_dims(const dg_handle* h, int* X, int* Y, int* Z)
{
    if (!h) return fail(DG_ERR_INVALID, "dg_dims: null handle");
    const dg::MeshHost& m = h->s.mesh;
    if (X) *X = m.E[0] * m.K;
    if (Y) *Y = m.E[1] * m.K;
    if (Z) *Z = m.E[2] * m.K;
    return DG_OK;
}

int dg_get_state(dg_handle* h, double* drho, double* vel)
{
    if (!h) return fail(DG_ERR_INVALID, "dg_get_state: null handle");
    return h->s.pack_out(h->s.state_ptr(), drho, vel);
}

int dg_set_state(dg_handle* h, const double* drho, const double* vel)
{
    if (!h || !drho || !vel) return fail(DG_ERR_INVALID, "dg_set_state: null argument");
    return h->s.unpack_in(drho, vel);
}

int dg_set_state_async(dg_handle* h, const double* drho, const double* vel)
{
    if (!h || !drho || !vel) return fail(DG_ERR_INVALID, "dg_set_state_async: null argument");
    return h->s.set_state_async(drho, vel);
}

int dg_step_get_state_async(dg_handle* h, double dt, double* drho, double* vel)
{
    if (!h || !drho || !vel) return fail(DG_ERR_INVALID, "dg_step_get_state_async: null argument");
    if (!std::isfinite(dt)) return fail(DG_ERR_INVALID, "dg_step_get_state_async: bad dt");
    return h->s.step_get_async(dt, drho, vel);
}

int dg_get_state_async(dg_handle* h, double* drho, double* vel)
{
    if (!h || (!drho && !vel)) return fail(DG_ERR_INVALID, "dg_get_state_async: null argument");
    return h->s.get_state_async(drho, vel);
}

int dg_eval_rhs(dg_handle* h, double* drho, double* vel)
{
    if (!h) return fail(DG_ERR_INVALID, "dg_eval_rhs: null handle");
    return h->s.eval_rhs(drho, vel);
}

int dg_get_grid(dg_handle* h, double* coords, double* sigma)
{
    if (!h) return fail(DG_ERR_INVALID, "dg_get_grid: null handle");
    const dg::MeshHost& m = h->s.mesh;
    const int K3 = m.K * m.K * m.K;
    const size_t gs = h->s.gsize();
    std::vector<double> x;
    for (int e = 0; e < m.n_elem; e++) {
        m.node_coords(h->s.p, h->s.op, e, x);
        for (int n = 0; n < K3; n++) {
            size_t g = dg::grid_offset(m, e, n);
            if (coords)
                for (int a = 0; a < 3; a++) coords[a * gs + g] = x[a * K3 + n];
            if (sigma) sigma[g] = m.sigma[e];
        }
    }
    return DG_OK;
}

double dg_time(const dg_handle* h) { return h ? h->s.t : 0.0; }

long long dg_launch_count(const dg_handle* h) { return h ? h->s.launches : 0; }

int dg_probe_set(dg_handle* h, int n, const double* xyz)
{
    if (!h || n < 0 || (n > 0 && !xyz)) return fail(DG_ERR_INVALID, "dg_probe_set: bad argument");
    Solver& s = h->s;
    cudaError_t e = cudaStreamSynchronize(s.stream);
    if (e != cudaSuccess) return fail(DG_ERR_CUDA, std::string("cudaStreamSynchronize: ") + cudaGetErrorString(e));
    const dg::MeshHost& m = s.mesh;
    const int K = m.K, K3 = K * K * K;
    std::vector<long long> off(n);
    std::vector<double> x;
    for (int i = 0; i < n; i++) {
        // the element containing the point (clamped to the mesh), then its nearest node
        int g[3];
        for (int a = 0; a < 3; a++) {
            const double r = (xyz[3 * i + a] - s.p.corner[a]) / s.p.elem_width[a];
            g[a] = std::min(m.E[a] - 1, std::max(0, (int)std::floor(r)));
        }
        const int el = m.elem_index(g);
        m.node_coords(s.p, s.op, el, x);
        int best = 0;
        double bd = 1e300;
        for (int nn = 0; nn < K3; nn++) {
            double d2 = 0;
            for (int a = 0; a < 3; a++) d2 += (x[a * K3 + nn] - xyz[3 * i + a]) * (x[a * K3 + nn] - xyz[3 * i + a]);
            if (d2 < bd) {
                bd = d2;
                best = nn;
            }
        }
        off[i] = (long long)el * m.NP + best;
    }
    if (s.d_probe_off) cudaFree(s.d_probe_off);
    if (s.d_probe_rec) cudaFree(s.d_probe_rec);
    s.d_probe_off = nullptr;
    s.d_probe_rec = nullptr;
    s.probe_cap = s.probe_steps = 0;
    s.probe_t.clear();
    s.n_probe = n;
    if (n == 0) return DG_OK;
    e = cudaMalloc(&s.d_probe_off, n * sizeof(long long));
    if (e != cudaSuccess) return fail(DG_ERR_CUDA, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    e = cudaMemcpy(s.d_probe_off, off.data(), n * sizeof(long long), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return fail(DG_ERR_CUDA, std::string("cudaMemcpy: ") + cudaGetErrorString(e));
    return s.probe_reserve(1024);
}

int dg_probe_get(dg_handle* h, double* t, double* p, int max_steps, int* steps)
{
    if (!h || max_steps < 0) return fail(DG_ERR_INVALID, "dg_probe_get: bad argument");
    Solver& s = h->s;
    const long long ns = std::min<long long>(s.probe_steps, max_steps);
    if (p && ns > 0 && s.n_probe > 0) {
        cudaError_t e = cudaMemcpyAsync(p, s.d_probe_rec, (size_t)ns * s.n_probe * sizeof(double),
                                        cudaMemcpyDeviceToHost, s.stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s.stream);
        if (e != cudaSuccess) return fail(DG_ERR_CUDA, std::string("dg_probe_get: ") + cudaGetErrorString(e));
    }
    if (t)
        for (long long i = 0; i < ns; i++) t[i] = s.probe_t[i];
    if (steps) *steps = (int)s.probe_steps;
    return DG_OK;
}

int dg_stream(dg_handle* h, void** stream)
{
    if (!h || !stream) return fail(DG_ERR_INVALID, "dg_stream: null argument");
    *stream = (void*)h->s.stream;
    return DG_OK;
}

int dg_profile(dg_handle* h, int enable)
{
    if (!h) return fail(DG_ERR_INVALID, "dg_profile: null handle");
    cudaError_t e = cudaStreamSynchronize(h->s.stream);
    if (e != cudaSuccess) return fail(DG_ERR_CUDA, std::string("cudaStreamSynchronize: ") + cudaGetErrorString(e));
    if (enable) h->s.prof_reset();
    h->s.profiling = enable != 0;
    return DG_OK;
}

int dg_kernel_stats(dg_handle* h, int k, long long* launches, double* ms, double* bytes, double* flops)
{
    if (!h || k < 0 || k > 1) return fail(DG_ERR_INVALID, "dg_kernel_stats: bad argument");
    cudaError_t e = cudaStreamSynchronize(h->s.stream);
    if (e != cudaSuccess) return fail(DG_ERR_CUDA, std::string("cudaStreamSynchronize: ") + cudaGetErrorString(e));
    const Solver::KernelStat& st = h->s.kstat[k];
    double total = 0.0;
    for (const auto& pr : st.ev) {
        float t = 0.f;
        if (cudaEventElapsedTime(&t, pr.first, pr.second) == cudaSuccess) total += t;
    }
    if (launches) *launches = st.launches;
    if (ms) *ms = total;
    if (bytes) *bytes = st.bytes;
    if (flops) *flops = st.flops;
    return DG_OK;
}

int dg_state_device(dg_handle* h, void* base[4], size_t* node_stride, int* n_elem)
{
    if (!h || !base) return fail(DG_ERR_INVALID, "dg_state_device: null argument");
    // the caller may write the state: the next FP64 stage evaluates the volume
    // fluxes from it instead of reading the ones cached by the last stage
    h->s.flux_valid = false;
    h->s.wait_pack(h->s.stream, h->s.state_ptr());
    const size_t es = h->s.fp64() ? 8 : 4;
    char* b = (char*)h->s.state_ptr();
    for (int f = 0; f < 4; f++) base[f] = b + (size_t)f * h->s.mesh.fstride() * es;
    if (node_stride) *node_stride = (size_t)h->s.mesh.NP;
    if (n_elem) *n_elem = h->s.mesh.n_elem;
    return DG_OK;
}

const char* dg_last_error(void) { return dg::g_last_error.c_str(); }

int dg_write_basis_files(const char* folder, int kmax, int lumped_mass)
{
    if (!folder || kmax < 2 || kmax > 10) return fail(DG_ERR_INVALID, "dg_write_basis_files: bad argument");
    std::string err = dg::write_coeff_files(folder, kmax);
    if (err.empty()) err = dg::write_matrix_file(std::string(folder) + "/matrices.txt", kmax - 1, lumped_mass != 0);
    if (!err.empty()) return fail(DG_ERR_IO, err);
    return DG_OK;
}

int dg_line_operators(int order, int lumped_mass, const char* matrix_file, const char* coeff_file, double* mass,
                      double* stiff, double* deriv, double* lift0, double* liftN, double* zeros)
{
    dg::LineOperators op;
    std::string err = dg::build_line_operators(order, lumped_mass != 0, matrix_file ? matrix_file : "",
                                               coeff_file ? coeff_file : "", op);
    if (!err.empty()) return fail(err.find("Opening") == 0 ? DG_ERR_IO : DG_ERR_INVALID, err);
    const int K = order + 1;
    if (mass) std::memcpy(mass, op.mass.data(), sizeof(double) * K * K);
    if (stiff) std::memcpy(stiff, op.stiff.data(), sizeof(double) * K * K);
    if (deriv) std::memcpy(deriv, op.deriv.data(), sizeof(double) * K * K);
    if (lift0) std::memcpy(lift0, op.lift0.data(), sizeof(double) * K);
    if (liftN) std::memcpy(liftN, op.liftN.data(), sizeof(double) * K);
    if (zeros) std::memcpy(zeros, op.zeros.data(), sizeof(double) * K);
    return DG_OK;
}

}  // extern "C"
