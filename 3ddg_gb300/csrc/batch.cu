// Batched form (dg_batch_*): many independent FP32 problems of uneven
// element counts and orders advanced together by the persistent stage kernels
// of batch_kernels.cuh (one per order, each group of problems sharing an
// operator on its own branch), one captured CUDA graph per RK step, tile sizes
// chosen per order by an autotuner.  The serving form (serve.cu) drives the same
// object, adding and removing problems as requests arrive and finish.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "batch_internal.h"
#include "batch_kernels.cuh"
#include "dg3d.h"
#include "dg_kernels.cuh"
#include "mesh.h"
#include "solver_internal.h"

namespace dg {



#define DGB_CUDA(call)                                                                         \
    do {                                                                                       \
        cudaError_t _e = (call);                                                               \
        if (_e != cudaSuccess)                                                                 \
            return fail(DG_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(_e));    \
    } while (0)

size_t batch_problem_bytes(const dg_params& p)
{
    const int K = p.order + 1;
    const size_t np = (size_t)(K * K * K + 7) / 8 * 8;
    size_t ne = 1;
    for (int a = 0; a < 3; a++) ne *= (size_t)p.num_blocks[a] * p.num_elements[a];
    return ne * np * 23 * sizeof(float) + ne * (6 * sizeof(int) + sizeof(float));
}

namespace {

constexpr size_t kAlign = 256;
inline size_t align_up(size_t n) { return (n + kAlign - 1) / kAlign * kAlign; }

template <int K>
void fill_ops(BatchProblem& P, const LineOperators& op, const dg_params& p)
{
    const double w1[3] = {1.0, 1.0, 1.0};
    const OpConst<double, K> C =
        make_stage_const<double, K>(1.0, op.deriv.data(), op.lift0.data(), op.liftN.data(), w1, p.rho0, p.c0,
                                    p.b_over_a, p.diff_const);
    for (int i = 0; i < K; i++) {
        for (int j = 0; j < K; j++) P.rows[i][j] = (float)op.deriv[i * K + j];
        P.rows[i][K] = (float)op.lift0[i];
        P.rows[i][K + 1] = (float)op.liftN[i];
    }
    for (int s = 0; s < 2; s++)
        for (int i = 0; i < 4; i++) {
            P.cM[s][i] = (float)C.cM[0][s][i];
            P.cA[s][i] = (float)C.cA[0][s][i];
        }
    P.k1 = (float)C.k1;
    P.k2 = (float)C.k2;
    P.r0 = (float)C.r0;
    P.inv_c2 = (float)C.inv_c2;
    P.inv_z = (float)C.inv_z;
    P.linear_mass = C.linear_mass;
}

}  // namespace

// ------------------------------------------------------------ PinnedPool
PinnedPool::Block* PinnedPool::acquire(size_t bytes, std::string& err)
{
    std::lock_guard<std::mutex> lock(mu);
    Block* best = nullptr;
    for (auto& b : blocks) {
        if (b->busy || b->cap < bytes) continue;
        if (b->ev_pending) {
            const cudaError_t q = cudaEventQuery(b->ev);
            if (q == cudaErrorNotReady) {
                (void)cudaGetLastError();
                continue;
            }
            if (q != cudaSuccess) {
                err = std::string("cudaEventQuery: ") + cudaGetErrorString(q);
                return nullptr;
            }
            b->ev_pending = false;
        }
        if (!best || b->cap < best->cap) best = b.get();
    }
    if (!best) {
        auto nb = std::make_unique<Block>();
        const size_t mib = (size_t)1 << 20;
        nb->cap = (std::max(bytes, mib) + mib - 1) / mib * mib;
        cudaError_t e = cudaHostAlloc(&nb->ptr, nb->cap, cudaHostAllocPortable);
        if (e != cudaSuccess) {
            err = std::string("cudaHostAlloc: ") + cudaGetErrorString(e);
            return nullptr;
        }
        e = cudaEventCreateWithFlags(&nb->ev, cudaEventDisableTiming);
        if (e != cudaSuccess) {
            cudaFreeHost(nb->ptr);
            err = std::string("cudaEventCreate: ") + cudaGetErrorString(e);
            return nullptr;
        }
        best = nb.get();
        blocks.push_back(std::move(nb));
    }
    best->busy = true;
    return best;
}

void PinnedPool::release(Block* b, cudaStream_t after)
{
    if (!b) return;
    std::lock_guard<std::mutex> lock(mu);
    b->ev_pending = cudaEventRecord(b->ev, after) == cudaSuccess;
    if (!b->ev_pending) {
        // the stream is unusable: keep the block out of circulation
        (void)cudaGetLastError();
        return;
    }
    b->busy = false;
}

void PinnedPool::release_now(Block* b)
{
    if (!b) return;
    std::lock_guard<std::mutex> lock(mu);
    b->busy = false;
}

PinnedPool::~PinnedPool()
{
    for (auto& b : blocks) {
        if (b->ev) {
            cudaEventSynchronize(b->ev);
            cudaEventDestroy(b->ev);
        }
        if (b->ptr) cudaFreeHost(b->ptr);
    }
}

Batch::Prepared::~Prepared()
{
    if (pool && host) pool->release_now(host);
}

// ------------------------------------------------------------ Batch
std::string Batch::validate(const dg_params& p)
{
    std::string err = validate_params(p);
    if (!err.empty()) return err;
    if (p.order > BATCH_KMAX - 1) return "the batched form supports ORDER 1.." + std::to_string(BATCH_KMAX - 1);
    return "";
}

int Batch::init(int device_capacity)
{
    DGB_CUDA(cudaGetDevice(&device));
    DGB_CUDA(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
    for (int i = 0; i < kBranches; i++) {
        DGB_CUDA(cudaStreamCreateWithFlags(&branch[i], cudaStreamNonBlocking));
        DGB_CUDA(cudaEventCreateWithFlags(&join_ev[i], cudaEventDisableTiming));
    }
    DGB_CUDA(cudaEventCreateWithFlags(&fork_ev, cudaEventDisableTiming));
    cudaDeviceProp prop;
    DGB_CUDA(cudaGetDeviceProperties(&prop, device));
    num_sms = prop.multiProcessorCount;
    DGB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_k[2][0], batch_stage_kernel<2, 0>, bthreads_of(2), 0));
    DGB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_k[2][1], batch_stage_kernel<2, 1>, bthreads_of(2), 0));
    DGB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_k[3][0], batch_stage_kernel<3, 0>, bthreads_of(3), 0));
    DGB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_k[3][1], batch_stage_kernel<3, 1>, bthreads_of(3), 0));
    DGB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_k[4][0], batch_stage_kernel<4, 0>, bthreads_of(4), 0));
    DGB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_k[4][1], batch_stage_kernel<4, 1>, bthreads_of(4), 0));
    DGB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_k[5][0], batch_stage_kernel<5, 0>, bthreads_of(5), 0));
    DGB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_k[5][1], batch_stage_kernel<5, 1>, bthreads_of(5), 0));
    DGB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_k[6][0], batch_stage_kernel<6, 0>, bthreads_of(6), 0));
    DGB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_k[6][1], batch_stage_kernel<6, 1>, bthreads_of(6), 0));
    max_ctas_per_sm = 1;
    for (int k = 2; k <= BATCH_KMAX; k++) {
        for (int ph = 0; ph < 2; ph++) {
            occ_k[k][ph] = std::max(1, occ_k[k][ph]);
            max_ctas_per_sm = std::max(max_ctas_per_sm, occ_k[k][ph]);
        }
    }
    ctas_per_sm = max_ctas_per_sm;
    // a pool of this device's memory that keeps what is freed for reuse
    cudaMemPoolProps props;
    std::memset(&props, 0, sizeof props);
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = device;
    DGB_CUDA(cudaMemPoolCreate(&pool, &props));
    unsigned long long keep = ~0ull;
    DGB_CUDA(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep));
    capacity = std::max(16, device_capacity);
    DGB_CUDA(cudaMallocFromPoolAsync((void**)&d_probs, capacity * sizeof(BatchProblem), pool, stream));
    DGB_CUDA(cudaStreamSynchronize(stream));
    // Default tile sizes: the autotuner's choice on the 256-instance batch of
    // uneven problems (32, 64, 16 and 8 elements per tile at K = 3, 4, 5, 6),
    // which a batch that is not tuned itself (a server's) starts from.
    for (int k = 0; k <= BATCH_KMAX; k++) passes[k] = 4;
    passes[4] = 16;
    passes[5] = 8;
    passes[6] = 8;
    return DG_OK;
}

int Batch::prepare(const dg_params& p, double dt, int steps, const char* matrix_file, const char* coeff_file,
                   Prepared& out)
{
    std::string err = validate(p);
    if (!err.empty()) return fail(DG_ERR_INVALID, err);
    if (!(dt > 0.0) || steps < 1) return fail(DG_ERR_INVALID, "batch: dt must be > 0 and steps >= 1");
    LineOperators op;
    const std::string key = std::to_string(p.order) + "|" + std::to_string(p.lumped_mass) + "|" +
                            (matrix_file ? matrix_file : "") + "|" + (coeff_file ? coeff_file : "");
    {
        std::lock_guard<std::mutex> lock(op_mu);
        auto it = op_cache.find(key);
        if (it == op_cache.end()) {
            err = build_line_operators(p.order, p.lumped_mass != 0, matrix_file ? matrix_file : "",
                                       coeff_file ? coeff_file : "", op);
            if (!err.empty()) return fail(err.find("Opening") == 0 ? DG_ERR_IO : DG_ERR_INVALID, err);
            op_cache[key] = op;
        } else {
            op = it->second;
        }
    }
    MeshHost m;
    err = build_mesh(p, op, m, false);
    if (!err.empty()) return fail(DG_ERR_INVALID, err);

    Entry& E = out.E;
    E.op_key = key;
    E.p = p;
    E.dt = dt;
    E.steps = steps;
    E.K = m.K;
    E.np = m.NP;
    E.n_elem = m.n_elem;
    for (int a = 0; a < 3; a++) {
        E.dims[a] = m.E[a] * m.K;
        E.nb[a] = m.nb[a];
        E.ne[a] = m.ne[a];
    }
    E.fs = m.fstride();
    out.data_bytes = align_up(E.fs * 23 * sizeof(float));
    out.nbr_bytes = align_up(m.nbr.size() * sizeof(int));
    E.chunk_bytes = out.data_bytes + out.nbr_bytes + align_up(m.sigma.size() * sizeof(float));

    // page-locked staging: nbr | sigma | [state0]
    out.has_state0 = !m.state0.empty();
    out.sigma_off = out.nbr_bytes;
    out.state_off = out.sigma_off + align_up(m.sigma.size() * sizeof(float));
    const size_t hbytes = out.state_off + (out.has_state0 ? 4 * E.fs * sizeof(float) : 0);
    out.pool = &pinned;
    out.host = pinned.acquire(hbytes, err);
    if (!out.host) return fail(DG_ERR_CUDA, "batch: " + err);
    unsigned char* h = (unsigned char*)out.host->ptr;
    int* hn = (int*)h;
    for (size_t i = 0; i < m.nbr.size(); i++) hn[i] = m.nbr[i] >= 0 ? m.nbr[i] : -1 - m.bnd_face[-1 - m.nbr[i]];
    float* hs = (float*)(h + out.sigma_off);
    for (size_t i = 0; i < m.sigma.size(); i++) hs[i] = (float)m.sigma[i];
    if (out.has_state0) {
        float* h0 = (float*)(h + out.state_off);
        for (size_t i = 0; i < 4 * E.fs; i++) h0[i] = (float)m.state0[i];
    }

    BatchProblem& P = E.desc;
    std::memset(&P, 0, sizeof P);
    P.K = m.K;
    P.np = m.NP;
    P.n_elem = m.n_elem;
    P.src_face = p.src_face;
    P.active = 1;
    P.cur = 0;
    P.steps_left = steps;
    P.fs = E.fs;
    switch (m.K) {
    case 2: fill_ops<2>(P, op, p); break;
    case 3: fill_ops<3>(P, op, p); break;
    case 4: fill_ops<4>(P, op, p); break;
    case 5: fill_ops<5>(P, op, p); break;
    case 6: fill_ops<6>(P, op, p); break;
    }
    for (int a = 0; a < 3; a++) {
        P.invw[a] = (float)(1.0 / p.elem_width[a]);
        P.gscale[a] = (float)(p.eval_diff ? p.diff_const / p.elem_width[a] : 0.0);
    }
    const double w23 = p.rk_exact ? 2.0 / 3.0 : (double)(2.0f / 3.0f);
    const double w13 = p.rk_exact ? 1.0 / 3.0 : (double)(1.0f / 3.0f);
    P.ca[0] = (float)dt;
    P.ca[1] = (float)(dt * .25);
    P.ca[2] = (float)(dt * 2.0 / 3.0);
    P.cb[0] = 0.f;
    P.cb[1] = .25f;
    P.cb[2] = (float)w23;
    P.eps = (float)(w23 + w13 - 1.0);
    if (!p.eval_advect) {
        P.k1 = P.k2 = 0.f;
        P.r0 = 0.f;
        P.linear_mass = 1;
        std::memset(P.cM, 0, sizeof P.cM);
        std::memset(P.cA, 0, sizeof P.cA);
    }
    P.t = 0.0;
    P.dt = dt;
    P.src_amp = p.src_amp;
    P.src_freq = p.src_freq;
    P.src_T = p.src_face >= 0 ? p.src_cycles / p.src_freq : 0.0;
    P.src_phase = p.src_phase;
    return DG_OK;
}

int Batch::commit(Prepared& pr, int* index)
{
    if (!pr.host) return fail(DG_ERR_STATE, "batch: problem not prepared");
    Entry E = pr.E;
    // the problem's memory first, so that a failed admission takes no slot
    DGB_CUDA(cudaMallocFromPoolAsync(&E.chunk, E.chunk_bytes, pool, stream));
    int slot;
    if (!free_slots.empty()) {
        slot = free_slots.back();
        free_slots.pop_back();
    } else {
        if (slot_hi >= capacity) {
            // grow the descriptor array in stream order
            const int ncap = capacity * 2;
            BatchProblem* nd = nullptr;
            cudaError_t e = cudaMallocFromPoolAsync((void**)&nd, ncap * sizeof(BatchProblem), pool, stream);
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(nd, d_probs, slot_hi * sizeof(BatchProblem), cudaMemcpyDeviceToDevice, stream);
            if (e != cudaSuccess) {
                if (nd) cudaFreeAsync(nd, stream);
                cudaFreeAsync(E.chunk, stream);
                return fail(DG_ERR_CUDA, std::string("batch: descriptor array: ") + cudaGetErrorString(e));
            }
            DGB_CUDA(cudaFreeAsync(d_probs, stream));
            d_probs = nd;
            capacity = ncap;
            graph_stale = true;
        }
        slot = slot_hi++;
    }
    unsigned char* c = (unsigned char*)E.chunk;
    E.data = c;
    E.nbr = (int*)(c + pr.data_bytes);
    E.sigma = (float*)(c + pr.data_bytes + pr.nbr_bytes);
    const unsigned char* h = (const unsigned char*)pr.host->ptr;
    DGB_CUDA(cudaMemsetAsync(E.data, 0, E.fs * 23 * sizeof(float), stream));
    DGB_CUDA(cudaMemcpyAsync(E.nbr, h, (size_t)E.n_elem * 6 * sizeof(int), cudaMemcpyHostToDevice, stream));
    DGB_CUDA(cudaMemcpyAsync(E.sigma, h + pr.sigma_off, (size_t)E.n_elem * sizeof(float), cudaMemcpyHostToDevice,
                             stream));
    if (pr.has_state0)
        DGB_CUDA(cudaMemcpyAsync(E.data, h + pr.state_off, 4 * E.fs * sizeof(float), cudaMemcpyHostToDevice, stream));
    pinned.release(pr.host, stream);
    pr.host = nullptr;

    BatchProblem& P = E.desc;
    float* base = (float*)E.data;
    P.u[0] = base;
    P.u[1] = base + 4 * E.fs;
    P.comp = base + 8 * E.fs;
    P.d[0] = base + 12 * E.fs;
    P.d[1] = base + 16 * E.fs;
    P.q = base + 20 * E.fs;
    P.nbr = E.nbr;
    P.sigma = E.sigma;
    batch_set_problem<<<1, 128, 0, stream>>>(d_probs + slot, P);
    DGB_CUDA(cudaGetLastError());
    E.slot = slot;
    E.id = next_id++;
    probs.push_back(E);
    if (index) *index = (int)probs.size() - 1;
    tiles_dirty = true;
    return DG_OK;
}

int Batch::add(const dg_params& p, double dt, int steps, const char* matrix_file, const char* coeff_file, int* index)
{
    Prepared pr;
    int rc = prepare(p, dt, steps, matrix_file, coeff_file, pr);
    if (rc) return rc;
    return commit(pr, index);
}

int Batch::remove(int i)
{
    if (i < 0 || i >= (int)probs.size()) return fail(DG_ERR_INVALID, "batch: bad problem index");
    Entry& E = probs[i];
    BatchProblem off;
    std::memset(&off, 0, sizeof off);
    batch_set_problem<<<1, 128, 0, stream>>>(d_probs + E.slot, off);
    DGB_CUDA(cudaGetLastError());
    DGB_CUDA(cudaFreeAsync(E.chunk, stream));
    free_slots.push_back(E.slot);
    probs.erase(probs.begin() + i);
    tiles_dirty = true;
    return DG_OK;
}

int Batch::enqueue_state_copy(int i, long long steps_done, PinnedPool::Block* dst)
{
    if (i < 0 || i >= (int)probs.size()) return fail(DG_ERR_INVALID, "batch: bad problem index");
    const Entry& E = probs[i];
    const size_t g = (size_t)E.n_elem * E.K * E.K * E.K;
    if (!dst || dst->cap < 4 * g * sizeof(double)) return fail(DG_ERR_INVALID, "batch: result block too small");
    double* st = nullptr;
    DGB_CUDA(cudaMallocFromPoolAsync((void**)&st, 4 * g * sizeof(double), pool, stream));
    GridMap gm;
    gm.K = E.K;
    for (int a = 0; a < 3; a++) {
        gm.nb[a] = E.nb[a];
        gm.ne[a] = E.ne[a];
        gm.E[a] = E.nb[a] * E.ne[a];
    }
    gm.elem_per_block = E.ne[0] * E.ne[1] * E.ne[2];
    // the state ping-pongs once per step, starting in u[0]
    const float* u = E.desc.u[steps_done & 1];
    pack_grid_kernel<float><<<304, 256, 0, stream>>>(u, E.fs, E.np, 4, gm, E.n_elem, st, g);
    DGB_CUDA(cudaGetLastError());
    DGB_CUDA(cudaMemcpyAsync(dst->ptr, st, 4 * g * sizeof(double), cudaMemcpyDeviceToHost, stream));
    DGB_CUDA(cudaFreeAsync(st, stream));
    return DG_OK;
}

void Batch::build_tiles()
{
    tiles.clear();
    groups.clear();
    // groups by order (largest first) and operator; within a group the
    // atomic tile counter hands out the tiles in order
    std::vector<int> order(probs.size());
    for (size_t i = 0; i < order.size(); i++) order[i] = (int)i;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
        if (probs[a].K != probs[b].K) return probs[a].K > probs[b].K;
        return probs[a].op_key < probs[b].op_key;
    });
    // Elements of each group (order and operator), so that a small group (few
    // problems in flight) gets tiles small enough for about two waves of its
    // persistent grid instead of leaving SMs idle; a large group keeps the
    // tuned tile size.
    std::vector<long long> group_elems;
    for (size_t n = 0; n < order.size(); n++) {
        const Entry& E = probs[order[n]];
        if (n == 0 || probs[order[n - 1]].K != E.K || probs[order[n - 1]].op_key != E.op_key)
            group_elems.push_back(0);
        group_elems.back() += E.n_elem;
    }
    int chunk = 0;
    for (size_t n = 0; n < order.size(); n++) {
        const int i = order[n];
        const Entry& E = probs[i];
        const int K = E.K;
        if (groups.empty() || groups.back().K != K || probs[order[n - 1]].op_key != E.op_key) {
            Group g;
            g.K = K;
            g.begin = g.end = (int)tiles.size();
            std::memcpy(g.ops.rows, E.desc.rows, sizeof g.ops.rows);
            groups.push_back(g);
            const long long waves2 = 2LL * num_sms * std::max(1, std::min(ctas_per_sm, occ_k[K][1]));
            const long long fit = (group_elems[groups.size() - 1] + bepb_of(K) * waves2 - 1) / (bepb_of(K) * waves2);
            chunk = bepb_of(K) * (int)std::max(1LL, std::min<long long>(std::max(1, passes[K]), fit));
        }
        for (int e0 = 0; e0 < E.n_elem; e0 += chunk) {
            BatchTile t;
            t.prob = E.slot;
            t.e0 = e0;
            t.count = std::min(chunk, E.n_elem - e0);
            t.K = K;
            tiles.push_back(t);
        }
        groups.back().end = (int)tiles.size();
    }
}

// Rebuild the tile list and upload it in stream order (after the steps
// already enqueued, which read the previous list); no synchronisation.
int Batch::upload_tiles()
{
    build_tiles();
    const int G = (int)groups.size();
    if (G > counter_groups) {
        // tile counters: [stage][group][phase]
        const int ng = std::max(G, std::max(8, 2 * counter_groups));
        int* nc = nullptr;
        DGB_CUDA(cudaMallocFromPoolAsync((void**)&nc, 3 * ng * 2 * sizeof(int), pool, stream));
        if (d_counters) DGB_CUDA(cudaFreeAsync(d_counters, stream));
        d_counters = nc;
        counter_groups = ng;
    }
    if ((int)tiles.size() > tile_capacity) {
        const int cap = std::max<int>((int)tiles.size(), 2 * tile_capacity);
        BatchTile* nt = nullptr;
        DGB_CUDA(cudaMallocFromPoolAsync((void**)&nt, cap * sizeof(BatchTile), pool, stream));
        if (d_tiles) DGB_CUDA(cudaFreeAsync(d_tiles, stream));
        d_tiles = nt;
        tile_capacity = cap;
    }
    if (!tiles.empty()) {
        std::string err;
        PinnedPool::Block* b = pinned.acquire(tiles.size() * sizeof(BatchTile), err);
        if (!b) return fail(DG_ERR_CUDA, "batch: " + err);
        std::memcpy(b->ptr, tiles.data(), tiles.size() * sizeof(BatchTile));
        cudaError_t e = cudaMemcpyAsync(d_tiles, b->ptr, tiles.size() * sizeof(BatchTile), cudaMemcpyHostToDevice,
                                        stream);
        pinned.release(b, stream);
        if (e != cudaSuccess) return fail(DG_ERR_CUDA, std::string("cudaMemcpyAsync: ") + cudaGetErrorString(e));
    }
    tiles_dirty = false;
    graph_stale = true;
    return DG_OK;
}

int Batch::launch_step()
{
    const int n = slot_hi;
    const int G = (int)groups.size();
    DGB_CUDA(cudaMemsetAsync(d_counters, 0, 3 * G * 2 * sizeof(int), stream));
    batch_step_begin<<<(n + 127) / 128, 128, 0, stream>>>(d_probs, n);
    launches += 2;
    // fork: group g runs its three stages on branch g % kBranches
    const int nb = std::min(G, (int)kBranches);
    DGB_CUDA(cudaEventRecord(fork_ev, stream));
    for (int b = 0; b < nb; b++) DGB_CUDA(cudaStreamWaitEvent(branch[b], fork_ev, 0));
    for (int g = 0; g < G; g++) {
        const Group& grp = groups[g];
        const int K = grp.K;
        cudaStream_t bs = branch[g % kBranches];
        for (int s = 0; s < 3; s++) {
            BatchArgs A;
            A.probs = d_probs;
            A.tiles = d_tiles;
            A.tile0 = grp.begin;
            A.n_tiles = grp.end - grp.begin;
            A.counters = d_counters + 2 * (s * G + g);
            A.stage = s;
            // persistent grid, but no more CTAs than the group has tiles: a small
            // group (few problems in flight) leaves room for the other branches
            for (int phase = 0; phase < 2; phase++) {
                const int grid =
                    std::max(1, std::min(num_sms * std::min(ctas_per_sm, occ_k[K][phase]), A.n_tiles));
                switch (K * 2 + phase) {
                case 4: batch_stage_kernel<2, 0><<<grid, bthreads_of(2), 0, bs>>>(A, grp.ops); break;
                case 5: batch_stage_kernel<2, 1><<<grid, bthreads_of(2), 0, bs>>>(A, grp.ops); break;
                case 6: batch_stage_kernel<3, 0><<<grid, bthreads_of(3), 0, bs>>>(A, grp.ops); break;
                case 7: batch_stage_kernel<3, 1><<<grid, bthreads_of(3), 0, bs>>>(A, grp.ops); break;
                case 8: batch_stage_kernel<4, 0><<<grid, bthreads_of(4), 0, bs>>>(A, grp.ops); break;
                case 9: batch_stage_kernel<4, 1><<<grid, bthreads_of(4), 0, bs>>>(A, grp.ops); break;
                case 10: batch_stage_kernel<5, 0><<<grid, bthreads_of(5), 0, bs>>>(A, grp.ops); break;
                case 11: batch_stage_kernel<5, 1><<<grid, bthreads_of(5), 0, bs>>>(A, grp.ops); break;
                case 12: batch_stage_kernel<6, 0><<<grid, bthreads_of(6), 0, bs>>>(A, grp.ops); break;
                case 13: batch_stage_kernel<6, 1><<<grid, bthreads_of(6), 0, bs>>>(A, grp.ops); break;
                }
                DGB_CUDA(cudaGetLastError());
                launches++;
            }
        }
    }
    // join
    for (int b = 0; b < nb; b++) {
        DGB_CUDA(cudaEventRecord(join_ev[b], branch[b]));
        DGB_CUDA(cudaStreamWaitEvent(stream, join_ev[b], 0));
    }
    batch_step_end<<<(n + 127) / 128, 128, 0, stream>>>(d_probs, n);
    DGB_CUDA(cudaGetLastError());
    return DG_OK;
}

int Batch::step(int nsteps)
{
    if (probs.empty()) return DG_OK;
    if (tiles_dirty) {
        int rc = upload_tiles();
        if (rc) return rc;
    }
    if (use_graph && (graph_stale || !graph)) {
        // capture the step; update the instantiated graph in place when its
        // shape allows, else instantiate anew
        cudaGraph_t g = nullptr;
        DGB_CUDA(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
        const long long before = launches;
        int rc = launch_step();
        step_kernels = launches - before;  // kernels per replay; nothing ran during capture
        launches = before;
        cudaError_t ec = cudaStreamEndCapture(stream, &g);
        if (rc || ec != cudaSuccess) {
            if (g) cudaGraphDestroy(g);
            cudaGetLastError();
            if (graph) cudaGraphExecDestroy(graph);
            graph = nullptr;
            use_graph = false;  // capture unsupported here: launch directly
        } else {
            if (graph) {
                cudaGraphExecUpdateResultInfo info;
                if (cudaGraphExecUpdate(graph, g, &info) != cudaSuccess) {
                    cudaGetLastError();
                    cudaGraphExecDestroy(graph);
                    graph = nullptr;
                }
            }
            if (!graph) {
                cudaError_t ei = cudaGraphInstantiate(&graph, g, 0);
                if (ei != cudaSuccess) {
                    graph = nullptr;
                    use_graph = false;
                    cudaGetLastError();
                }
            }
            cudaGraphDestroy(g);
        }
        graph_stale = false;
    }
    for (int i = 0; i < nsteps; i++) {
        if (graph) {
            DGB_CUDA(cudaGraphLaunch(graph, stream));
            launches += step_kernels;
        } else {
            int rc = launch_step();
            if (rc) return rc;
        }
    }
    return DG_OK;
}

int Batch::sync_descs()
{
    if (probs.empty()) return DG_OK;
    std::vector<BatchProblem> h(slot_hi);
    DGB_CUDA(cudaMemcpyAsync(h.data(), d_probs, h.size() * sizeof(BatchProblem), cudaMemcpyDeviceToHost, stream));
    DGB_CUDA(cudaStreamSynchronize(stream));
    for (Entry& E : probs) E.desc = h[E.slot];
    return DG_OK;
}

int Batch::get_state(int i, double* drho, double* vel)
{
    if (i < 0 || i >= (int)probs.size()) return fail(DG_ERR_INVALID, "batch: bad problem index");
    int rc = sync_descs();
    if (rc) return rc;
    Entry& E = probs[i];
    const size_t g = (size_t)E.n_elem * E.K * E.K * E.K;
    double* st = nullptr;
    DGB_CUDA(cudaMallocFromPoolAsync((void**)&st, 4 * g * sizeof(double), pool, stream));
    GridMap gm;
    gm.K = E.K;
    for (int a = 0; a < 3; a++) {
        gm.nb[a] = E.nb[a];
        gm.ne[a] = E.ne[a];
        gm.E[a] = E.nb[a] * E.ne[a];
    }
    gm.elem_per_block = E.ne[0] * E.ne[1] * E.ne[2];
    const float* u = E.desc.u[E.desc.cur];
    pack_grid_kernel<float><<<304, 256, 0, stream>>>(u, E.fs, E.np, 4, gm, E.n_elem, st, g);
    DGB_CUDA(cudaGetLastError());
    if (drho) DGB_CUDA(cudaMemcpyAsync(drho, st, g * sizeof(double), cudaMemcpyDeviceToHost, stream));
    if (vel) DGB_CUDA(cudaMemcpyAsync(vel, st + g, 3 * g * sizeof(double), cudaMemcpyDeviceToHost, stream));
    DGB_CUDA(cudaFreeAsync(st, stream));
    DGB_CUDA(cudaStreamSynchronize(stream));
    return DG_OK;
}

// Save / restore of every problem's time-dependent data, for the autotuner.
int Batch::snapshot(std::vector<std::vector<char>>& save)
{
    int rc = sync_descs();
    if (rc) return rc;
    save.resize(probs.size());
    for (size_t i = 0; i < probs.size(); i++) {
        const size_t bytes = probs[i].fs * 23 * sizeof(float);
        save[i].resize(bytes);
        DGB_CUDA(cudaMemcpyAsync(save[i].data(), probs[i].data, bytes, cudaMemcpyDeviceToHost, stream));
    }
    DGB_CUDA(cudaStreamSynchronize(stream));
    saved_desc.resize(probs.size());
    for (size_t i = 0; i < probs.size(); i++) saved_desc[i] = probs[i].desc;
    return DG_OK;
}

int Batch::restore(const std::vector<std::vector<char>>& save)
{
    for (size_t i = 0; i < probs.size(); i++) {
        DGB_CUDA(cudaMemcpyAsync(probs[i].data, save[i].data(), save[i].size(), cudaMemcpyHostToDevice, stream));
        batch_set_problem<<<1, 128, 0, stream>>>(d_probs + probs[i].slot, saved_desc[i]);
        DGB_CUDA(cudaGetLastError());
    }
    DGB_CUDA(cudaStreamSynchronize(stream));
    for (size_t i = 0; i < probs.size(); i++) probs[i].desc = saved_desc[i];
    return DG_OK;
}

int Batch::time_steps(int n, double* ms)
{
    cudaEvent_t a, b;
    DGB_CUDA(cudaEventCreate(&a));
    DGB_CUDA(cudaEventCreate(&b));
    int rc = step(1);  // warm: uploads, graph capture
    if (rc) return rc;
    DGB_CUDA(cudaEventRecord(a, stream));
    rc = step(n);
    if (rc) return rc;
    DGB_CUDA(cudaEventRecord(b, stream));
    DGB_CUDA(cudaEventSynchronize(b));
    float t = 0.f;
    DGB_CUDA(cudaEventElapsedTime(&t, a, b));
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    *ms = t / n;
    return DG_OK;
}

// Coordinate descent over the per-order tile size (passes of EPB elements per
// tile) and the persistent grid (CTAs per SM), timing real steps of this
// batch; the state is saved before and restored after.
int Batch::autotune(int trial_steps, std::string& report)
{
    if (probs.empty()) return DG_OK;
    std::vector<std::vector<char>> save;
    int rc = snapshot(save);
    if (rc) return rc;
    std::vector<int> orders;
    for (const Entry& E : probs)
        if (std::find(orders.begin(), orders.end(), E.K) == orders.end()) orders.push_back(E.K);
    std::sort(orders.begin(), orders.end());
    const int cand_pass[] = {1, 2, 4, 8, 16};
    double best = 0;
    tiles_dirty = true;
    rc = time_steps(trial_steps, &best);
    if (rc) return rc;
    report.clear();
    for (int round = 0; round < 2; round++) {
        for (int K : orders) {
            int keep = passes[K];
            for (int c : cand_pass) {
                if (c == keep) continue;
                passes[K] = c;
                tiles_dirty = true;
                double ms;
                if ((rc = restore(save))) return rc;
                if ((rc = time_steps(trial_steps, &ms))) return rc;
                if (ms < best * 0.995) {
                    best = ms;
                    keep = c;
                }
            }
            passes[K] = keep;
        }
        int keep_c = ctas_per_sm;
        for (int c = 1; c <= max_ctas_per_sm; c++) {
            if (c == keep_c) continue;
            ctas_per_sm = c;
            graph_stale = true;
            double ms;
            if ((rc = restore(save))) return rc;
            if ((rc = time_steps(trial_steps, &ms))) return rc;
            if (ms < best * 0.995) {
                best = ms;
                keep_c = c;
            }
        }
        ctas_per_sm = keep_c;
    }
    tiles_dirty = true;
    if ((rc = restore(save))) return rc;
    if ((rc = upload_tiles())) return rc;
    for (int K : orders) report += "K=" + std::to_string(K) + ":elems_per_tile=" + std::to_string(bepb_of(K) * passes[K]) + " ";
    report += "ctas_per_sm=" + std::to_string(ctas_per_sm) + " ms_per_step=" + std::to_string(best);
    return DG_OK;
}

size_t Batch::total_nodes() const
{
    size_t n = 0;
    for (const Entry& E : probs) n += (size_t)E.n_elem * E.K * E.K * E.K;
    return n;
}

Batch::~Batch()
{
    if (stream) cudaStreamSynchronize(stream);
    for (int i = 0; i < kBranches; i++) {
        if (branch[i]) {
            cudaStreamSynchronize(branch[i]);
            cudaStreamDestroy(branch[i]);
        }
        if (join_ev[i]) cudaEventDestroy(join_ev[i]);
    }
    if (fork_ev) cudaEventDestroy(fork_ev);
    if (graph) cudaGraphExecDestroy(graph);
    if (stream) {
        for (Entry& E : probs) cudaFreeAsync(E.chunk, stream);
        if (d_probs) cudaFreeAsync(d_probs, stream);
        if (d_tiles) cudaFreeAsync(d_tiles, stream);
        if (d_counters) cudaFreeAsync(d_counters, stream);
        cudaStreamSynchronize(stream);
    }
    if (pool) cudaMemPoolDestroy(pool);
    if (stream) cudaStreamDestroy(stream);
}

}  // namespace dg

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
struct dg_batch {
    dg::Batch b;
};

extern "C" {

int dg_batch_create(int n, const dg_params* params, const double* dt, const int* steps, const char* matrix_file,
                    const char* coeff_file, dg_batch** out)
{
    if (!out || n < 0 || (n > 0 && (!params || !dt || !steps)))
        return dg::fail(DG_ERR_INVALID, "dg_batch_create: bad argument");
    *out = nullptr;
    dg_batch* h = new (std::nothrow) dg_batch;
    if (!h) return dg::fail(DG_ERR_NOMEM, "dg_batch_create: host allocation failed");
    int rc = h->b.init(std::max(n, 16));
    for (int i = 0; rc == DG_OK && i < n; i++) rc = h->b.add(params[i], dt[i], steps[i], matrix_file, coeff_file, nullptr);
    if (rc) {
        delete h;
        return rc;
    }
    *out = h;
    return DG_OK;
}

int dg_batch_destroy(dg_batch* b)
{
    delete b;
    return DG_OK;
}

int dg_batch_step(dg_batch* b, int nsteps)
{
    if (!b || nsteps < 0) return dg::fail(DG_ERR_INVALID, "dg_batch_step: bad argument");
    return b->b.step(nsteps);
}

int dg_batch_synchronize(dg_batch* b)
{
    if (!b) return dg::fail(DG_ERR_INVALID, "dg_batch_synchronize: null handle");
    cudaError_t e = cudaStreamSynchronize(b->b.stream);
    if (e != cudaSuccess) return dg::fail(DG_ERR_CUDA, std::string("cudaStreamSynchronize: ") + cudaGetErrorString(e));
    return DG_OK;
}

int dg_batch_get_state(dg_batch* b, int i, double* drho, double* vel)
{
    if (!b) return dg::fail(DG_ERR_INVALID, "dg_batch_get_state: null handle");
    return b->b.get_state(i, drho, vel);
}

int dg_batch_info(dg_batch* b, int i, int* dims3, long long* steps_done, double* time)
{
    if (!b || i < 0 || i >= (int)b->b.probs.size()) return dg::fail(DG_ERR_INVALID, "dg_batch_info: bad argument");
    int rc = b->b.sync_descs();
    if (rc) return rc;
    const dg::Batch::Entry& E = b->b.probs[i];
    if (dims3)
        for (int a = 0; a < 3; a++) dims3[a] = E.dims[a];
    if (steps_done) *steps_done = E.desc.steps_done;
    if (time) *time = E.desc.t;
    return DG_OK;
}

long long dg_batch_total_nodes(const dg_batch* b) { return b ? (long long)b->b.total_nodes() : 0; }

int dg_batch_autotune(dg_batch* b, int trial_steps, char* report, size_t report_len)
{
    if (!b || trial_steps < 1) return dg::fail(DG_ERR_INVALID, "dg_batch_autotune: bad argument");
    std::string r;
    int rc = b->b.autotune(trial_steps, r);
    if (rc) return rc;
    if (report && report_len) {
        std::strncpy(report, r.c_str(), report_len - 1);
        report[report_len - 1] = 0;
    }
    return DG_OK;
}

int dg_batch_stream(dg_batch* b, void** stream)
{
    if (!b || !stream) return dg::fail(DG_ERR_INVALID, "dg_batch_stream: null argument");
    *stream = (void*)b->b.stream;
    return DG_OK;
}

long long dg_batch_launch_count(const dg_batch* b) { return b ? b->b.launches : 0; }

}  // extern "C"
