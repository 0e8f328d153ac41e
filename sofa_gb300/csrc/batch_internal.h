// Internal declarations shared by the batch engine (batch.cu) and the
// serving loop (server.cu).
#pragma once
#include <cuda_runtime.h>

#include <map>
#include <string>
#include <vector>

#include "../../include/sofa_gb300.h"
#include "mesh_layout.h"
#include "sgb_internal.h"
#include "variants.h"

namespace sgb {

// First-fit allocator over one device buffer (the batch's HBM budget).
struct Arena {
    char* base = nullptr;
    size_t size = 0;
    std::map<size_t, size_t> free_;  // offset -> length
    size_t used = 0;
    void reset(char* b, size_t n);
    bool alloc(size_t n, size_t* off);
    void release(size_t off, size_t n);
    size_t largest_free() const;
};

// A mesh whose host-side preparation (validation, element order, patch
// layout, gather tables) is done; admitting it only uploads and initialises.
struct PreparedMesh {
    int N = 0, E = 0, method = 1;
    sgb_scene_params P{};
    std::vector<double> rest;
    std::vector<int32_t> tets_store;
    HostLayout L;
    std::vector<int> rowptr, slots;
    std::vector<uint8_t> fixed;
    std::vector<double> node_mass, ext, Eh, nuh;
    size_t bytes = 0;
};

struct BatchMeshHost {
    bool active = false;
    size_t off = 0, bytes = 0;
    int n_nodes = 0, n_tets = 0, n_patches = 0, n_chunks = 0;
    long long steps = 0;
    std::vector<int> perm;
    BMeshDesc d{};  // host copy of the device descriptor's pointers/params
};

}  // namespace sgb

struct sgb_batch {
    const sgb::VariantOps* ops = nullptr;
    int precision = 0;
    size_t rs = 4;
    int pe = 512;  // elements per patch (shared-memory stride of the batch matvec)
    int fused_rhs = 2;  // forces and right-hand side: 2 by patches, 1 by elements (eforce_v), 0 four passes
    int max_slots = 0;
    int max_iterations = 0;
    sgb::Arena arena;
    char* arena_mem = nullptr;
    sgb::BMeshDesc* d_meshes = nullptr;
    std::vector<sgb::BatchMeshHost> slots;
    sgb::WorkItem* d_items[3] = {nullptr, nullptr, nullptr};
    int cap[3] = {0, 0, 0};
    int* d_counts = nullptr;
    int* d_err = nullptr;  // sticky device error flag: 1 = a bounded device wait ran out
    int counts_h[3] = {0, 0, 0};
    cudaStream_t stream = nullptr;
    cudaGraphExec_t graph = nullptr;
    bool graph_valid = false;
    int sms = 152;
    int grid_patch_v[4] = {152, 152, 152, 0};  // resident matvec CTAs per register-cap variant (kBatchMatvecMinb),
                                               // then those of the patch force / right-hand side pass
    sgb::BatchTiles tiles;                  // launch tiles (set by sgb_batch_tune / sgb_batch_set_tiles)
    double tune_default_ms = 0.0, tune_best_ms = 0.0;  // last tuning: step time of the default and chosen tiles
    int tune_trials = 0;                    // configurations timed by the last tuning (0: from the cache)
    size_t device_bytes = 0;
};


namespace sgb {
int prepare_mesh(const sgb_mesh_desc* m, int pe, size_t rs, PreparedMesh& out, int fused_rhs);
int batch_rhs_form(int fused_rhs, size_t rs);
int admit_prepared(sgb_batch* B, PreparedMesh& pm, int* slot);
}  // namespace sgb
