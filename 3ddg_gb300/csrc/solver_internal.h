// Internal state of one simulation handle (shared by the C-ABI translation
// units of libdg3d; not part of the public interface).
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <utility>
#include <vector>

#include "basis.h"
#include "dg3d.h"
#include "mesh.h"

namespace dg {

struct GridMap;
template <typename T>
struct FluxOut;

extern thread_local std::string g_last_error;
int fail(int code, const std::string& msg);
double burst_pressure(const dg_params& p, double t);

struct Solver {
    dg_params p{};
    LineOperators op;
    MeshHost mesh;
    int device = 0;
    cudaStream_t stream = nullptr;
    // FP64: buf[0] = U (stage 3 writes it in place), buf[1] = k1, buf[2] = k2.
    // FP32: buf[0], buf[1] = u ping-pong (buf[cur] current), buf[2] = Kahan
    //       compensation, buf[3] = d1, buf[4] = d2.
    void* buf[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
    void* qbuf = nullptr;       // LDG gradient, 3 fields
    double* staging = nullptr;  // 4 node-duplicated FP64 fields for host transfers
    int* d_nbr = nullptr;
    void* d_sigma = nullptr;
    void* d_bnd_ic = nullptr;
    void* d_bnd_ap = nullptr;
    int* d_bnd_src = nullptr;
    void* d_const = nullptr;  // per-launch operators: 3 RK stages, LDG gradient, bare RHS
    std::vector<char> h_const;  // host copy of d_const (for by-value kernel parameters)
    double* d_elem_b = nullptr;  // FP64: cb - ca sigma per element for the 3 RK stages
    // FP64 with advection: volume fluxes (f_mom, f_mass x, y, z) of the next
    // stage's input in d_flux[flux_cur], written by the stage that produced
    // it; flux_valid is false after anything else writes the state.
    double* d_flux[2] = {nullptr, nullptr};
    int flux_cur = 0;
    bool flux_valid = false;
    std::vector<double> h_elem_b;
    double const_dt = 0.0;
    int cur = 0;
    bool ic_live = false;
    double t = 0.0;
    long long steps_done = 0;
    long long launches = 0;

    // Optional per-launch event timing (dg_profile / dg_kernel_stats).
    struct KernelStat {
        std::vector<std::pair<cudaEvent_t, cudaEvent_t>> ev;
        long long launches = 0;
        double bytes = 0.0, flops = 0.0;
    };
    // Pressure probes: node offsets (element * NP + node) and the record.
    long long* d_probe_off = nullptr;
    int n_probe = 0;
    double* d_probe_rec = nullptr;  // [capacity][n_probe]
    long long probe_cap = 0, probe_steps = 0;
    std::vector<double> probe_t;
    int probe_reserve(long long steps);
    void probe_record();

    bool profiling = false;
    KernelStat kstat[2];
    std::vector<cudaEvent_t> event_pool;
    cudaEvent_t take_event();
    void prof_begin(int k, cudaEvent_t* a);
    void prof_end(int k, cudaEvent_t a, double bytes, double flops);
    void prof_reset();

    bool fp64() const { return p.precision == DG_PRECISION_FP64; }
    size_t gsize() const { return (size_t)mesh.n_elem * mesh.K * mesh.K * mesh.K; }
    size_t device_bytes() const;
    void* state_ptr() const;

    int init(const dg_params& prm, const char* matrix_file, const char* coeff_file);
    int step(double dt, int nsteps);
    int rk_stage_fp64(int s, double dt, double* rhs_only);
    int rk_stage_fp32(int s, double dt, float* rhs_only);
    int eval_rhs(double* drho, double* vel);
    int ensure_staging();
    int pack_out(const void* src, double* drho, double* vel);
    int unpack_in(const double* drho, const double* vel);
    int launch_unpack(const double* rho_d, const double* vel_d, bool on_device);
    template <typename T>
    cudaError_t launch_unpack_staged(T* state, const GridMap& g, const double* rho_d, const double* vel_d,
                                     const FluxOut<T>& fo, cudaStream_t st);

    // Asynchronous host transfers (dg_set_state_async / dg_get_state_async):
    // copy-engine streams and double-buffered device staging, so that one
    // step's upload and the previous step's download run under compute.  The
    // transposes between staging and the element-major state run on two
    // streams of their own (default priority): an upload is unpacked (xin) into a
    // spare state buffer (and, FP64 with advection, a spare flux buffer) that
    // the compute stream swaps in at the upload's place in the call sequence,
    // so the unpack runs under the step before; a download's pack (xout)
    // reads the state while the next steps compute.  A stream waits for a
    // pending pack only before it writes the buffer that pack reads (one
    // completion event per state buffer).
    cudaStream_t xin = nullptr, xout = nullptr;
    void* spare_u = nullptr;
    double* spare_f = nullptr;
    cudaEvent_t spare_ready = nullptr, spare_free = nullptr, step_done = nullptr;
    bool spare_free_recorded = false;
    struct PackEvent {
        const void* src = nullptr;
        cudaEvent_t ev = nullptr;
    };
    PackEvent pack_ev[3];  // FP32 has three state buffers (u ping-pong and the spare)
    void wait_pack(cudaStream_t st, const void* target);
    cudaStream_t copy_in = nullptr, copy_out = nullptr;
    double* astage_in[2] = {nullptr, nullptr};
    double* astage_out[2] = {nullptr, nullptr};
    cudaEvent_t in_ready[2] = {nullptr, nullptr}, in_free[2] = {nullptr, nullptr};
    cudaEvent_t out_ready[2] = {nullptr, nullptr}, out_free[2] = {nullptr, nullptr};
    int in_slot = 0, out_slot = 0;
    int ensure_async();
    int set_state_async(const double* drho, const double* vel);
    int get_state_async(double* drho, double* vel);
    int step_get_async(double dt, double* drho, double* vel);
    double* stage3_pack = nullptr;  // set by step_get_async: the last stage also packs its output here
    bool stage3_packed = false;      // it did
    int sync_all();
    ~Solver();
};

}  // namespace dg

// The opaque handle of the C ABI.
struct dg_handle {
    dg::Solver s;
};
