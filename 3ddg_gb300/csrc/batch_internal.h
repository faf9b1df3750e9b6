// Internal state of a batch of independent FP32 problems (dg_batch_*), shared
// by batch.cu and serve.cu; not part of the public interface.
#pragma once

#include <cuda_runtime.h>

#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "basis.h"
#include "batch_types.h"
#include "dg3d.h"

namespace dg {

// Device bytes one problem of the batched form holds (state, stages,
// compensation, gradient, face table, sigma).
size_t batch_problem_bytes(const dg_params& p);

// Page-locked host blocks for asynchronous copies.  A block handed back with
// release(b, stream) is reused only once the copies enqueued on that stream
// before the release have completed (an event per block), so the caller never
// waits for a copy to finish before reusing host memory.  Thread-safe.
class PinnedPool {
public:
    struct Block {
        void* ptr = nullptr;
        size_t cap = 0;
        cudaEvent_t ev = nullptr;
        bool busy = false, ev_pending = false;
    };
    Block* acquire(size_t bytes, std::string& err);
    void release(Block* b, cudaStream_t after);  // reusable once ``after`` passes this point
    void release_now(Block* b);                   // no copy in flight
    ~PinnedPool();

private:
    std::mutex mu;
    std::vector<std::unique_ptr<Block>> blocks;
};

struct Batch {
    struct Entry {
        dg_params p;
        double dt = 0.0;
        int steps = 0;
        int K = 0, np = 0, n_elem = 0;
        int dims[3] = {0, 0, 0};
        int nb[3] = {1, 1, 1}, ne[3] = {1, 1, 1};
        size_t fs = 0;
        int slot = -1;         // index of its descriptor in d_probs
        void* chunk = nullptr; // one pool allocation: data | nbr | sigma
        size_t chunk_bytes = 0;
        void* data = nullptr;  // 23 float fields: u0, u1, comp, d1, d2 (4 each), q (3)
        int* nbr = nullptr;
        float* sigma = nullptr;
        BatchProblem desc;     // host copy of the device descriptor
        std::string op_key;    // order | mass matrix | basis files
        long long id = 0;
    };

    // A problem built on the host (mesh tables, operators, descriptor) and
    // staged in page-locked memory, ready to be committed to the device
    // without host work or synchronisation.  prepare() may run on another
    // thread than the one driving the batch.
    struct Prepared {
        Entry E;
        PinnedPool* pool = nullptr;
        PinnedPool::Block* host = nullptr;  // nbr (6 n_elem int) | sigma (n_elem float) | [state0 (4 fs float)]
        size_t sigma_off = 0, state_off = 0;
        size_t data_bytes = 0, nbr_bytes = 0;  // offsets of nbr and sigma in the device chunk
        bool has_state0 = false;
        Prepared() = default;
        Prepared(const Prepared&) = delete;
        Prepared& operator=(const Prepared&) = delete;
        ~Prepared();
    };

    int device = 0;
    cudaStream_t stream = nullptr;
    // Device memory of the problems, stream-ordered (no device-wide
    // synchronisation when problems are added or removed).
    cudaMemPool_t pool = nullptr;
    PinnedPool pinned;
    // Branch streams: the groups' stage kernels run as parallel branches of
    // the step (each group's three stages in order on its branch), joined
    // before the step's end.
    static constexpr int kBranches = 6;
    cudaStream_t branch[kBranches] = {};
    cudaEvent_t fork_ev = nullptr, join_ev[kBranches] = {};
    int num_sms = 0, max_ctas_per_sm = 1, ctas_per_sm = 1;
    int occ_k[BATCH_KMAX + 1][2] = {};       // resident CTAs per SM of each order's kernel, per phase
    // Problems of one order sharing one operator (order, mass matrix, basis
    // files) form a group: one kernel launch per group and stage.
    struct Group {
        int K = 0, begin = 0, end = 0;  // tiles[begin .. end)
        BatchOps ops{};
    };
    std::vector<Group> groups;
    int counter_groups = 0;  // groups d_counters has room for
    long long step_kernels = 0;  // kernels in one captured step
    int passes[BATCH_KMAX + 1];  // autotuned: passes of EPB(K) elements per tile
    std::vector<Entry> probs;
    std::vector<BatchProblem> saved_desc;
    std::mutex op_mu;
    std::map<std::string, LineOperators> op_cache;
    // Descriptor slots: a problem keeps its slot for its whole life, a freed
    // slot holds an inactive descriptor; the step kernels walk slots
    // [0, slot_hi).
    BatchProblem* d_probs = nullptr;
    int capacity = 0, slot_hi = 0;
    std::vector<int> free_slots;
    std::vector<BatchTile> tiles;
    BatchTile* d_tiles = nullptr;
    int tile_capacity = 0;
    int* d_counters = nullptr;
    bool tiles_dirty = true;
    bool graph_stale = true;   // membership, tiles or launch shape changed since the capture
    bool use_graph = true;
    cudaGraphExec_t graph = nullptr;
    long long launches = 0;
    long long next_id = 1;

    static std::string validate(const dg_params& p);
    int init(int device_capacity);
    // Host part of add(): thread-safe, touches no device memory.
    int prepare(const dg_params& p, double dt, int steps, const char* matrix_file, const char* coeff_file,
                Prepared& out);
    // Device part: stream-ordered allocation, uploads and descriptor write.
    int commit(Prepared& pr, int* index);
    int add(const dg_params& p, double dt, int steps, const char* matrix_file, const char* coeff_file, int* index);
    // Stream-ordered removal: its memory returns to the pool after the work
    // already enqueued.
    int remove(int i);
    // Enqueue a copy of problem i's state after ``steps_done`` steps (the
    // dg_get_state layout, drho then vel, FP64) into a page-locked block.
    int enqueue_state_copy(int i, long long steps_done, PinnedPool::Block* dst);
    void build_tiles();
    int upload_tiles();
    int launch_step();
    int step(int nsteps);
    int sync_descs();
    int get_state(int i, double* drho, double* vel);
    int snapshot(std::vector<std::vector<char>>& save);
    int restore(const std::vector<std::vector<char>>& save);
    int time_steps(int n, double* ms);
    int autotune(int trial_steps, std::string& report);
    size_t total_nodes() const;
    ~Batch();
};

}  // namespace dg
