// Host-side element ordering and patch layout (mesh_layout.cu).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <vector>

namespace sgb {

struct HostLayout {
    std::vector<int> perm;        // storage position -> original element
    std::vector<int> inv;         // original element -> storage position
    std::vector<int> elem_start;  // n_patches + 1
    std::vector<int> node_start;  // n_patches + 1
    std::vector<int> lnode_gid;
    std::vector<int> lnode_info;
    std::vector<int> lrow;
    std::vector<uint16_t> lslots;
    std::vector<ushort4> lconn;
    std::vector<int> bnd_rowptr;
    int n_partials = 0, max_lnodes = 0, n_boundary = 0;
};

void build_patch_layout(int N, int E, const int32_t* tets, const double* pos, int pe, int pn_max, HostLayout& L);
void build_node_csr(int N, int E, const int32_t* tets, const std::vector<int>& inv, std::vector<int>& rowptr,
                    std::vector<int>& slots, int& max_valence);

}  // namespace sgb
