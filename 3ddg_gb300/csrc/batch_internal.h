// Internal state of a batch of independent FP32 problems (dg_batch_*), shared
// by batch.cu and serve.cpp; not part of the public interface.
#pragma once

#include <cuda_runtime.h>

#include <map>
#include <string>
#include <vector>

#include "basis.h"
#include "batch_types.h"
#include "dg3d.h"

namespace dg {

// Device bytes one problem of the batched form holds (state, stages,
// compensation, gradient, face table, sigma).
size_t batch_problem_bytes(const dg_params& p);

struct Batch {
    struct Entry {
        dg_params p;
        double dt = 0.0;
        int steps = 0;
        int K = 0, np = 0, n_elem = 0;
        int dims[3] = {0, 0, 0};
        int nb[3] = {1, 1, 1}, ne[3] = {1, 1, 1};
        size_t fs = 0;
        void* data = nullptr;  // 23 float fields: u0, u1, comp, d1, d2 (4 each), q (3)
        int* nbr = nullptr;
        float* sigma = nullptr;
        BatchProblem desc;     // host copy of the device descriptor
        std::string op_key;    // order | mass matrix | basis files
        long long id = 0;
    };

    int device = 0;
    cudaStream_t stream = nullptr;
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
    std::map<std::string, LineOperators> op_cache;
    BatchProblem* d_probs = nullptr;
    int capacity = 0;
    std::vector<BatchTile> tiles;
    BatchTile* d_tiles = nullptr;
    int tile_capacity = 0;
    int* d_counters = nullptr;
    bool tiles_dirty = true;
    bool use_graph = true;
    cudaGraphExec_t graph = nullptr;
    long long launches = 0;
    long long next_id = 1;

    static std::string validate(const dg_params& p);
    int init(int device_capacity);
    int add(const dg_params& p, double dt, int steps, const char* matrix_file, const char* coeff_file, int* index);
    int remove(int i);
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
