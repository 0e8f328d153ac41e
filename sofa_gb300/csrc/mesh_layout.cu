// Host-side construction of the element storage order and the patch layout
// used by the fused matvec kernel (see PatchView in sgb_internal.h).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <numeric>
#include <vector>

#include "mesh_layout.h"

namespace sgb {

static inline uint32_t spread10(uint32_t v)
{
    v &= 0x3ffu;
    v = (v | (v << 16)) & 0x030000FFu;
    v = (v | (v << 8)) & 0x0300F00Fu;
    v = (v | (v << 4)) & 0x030C30C3u;
    v = (v | (v << 2)) & 0x09249249u;
    return v;
}

void build_patch_layout(int N, int E, const int32_t* tets, const double* pos, int pe, int pn_max, HostLayout& L)
{
    // 1. Morton order of element centroids (one scale for all axes so that
    //    patches come out as compact blocks of cells)
    double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
    for (int n = 0; n < N; ++n)
        for (int k = 0; k < 3; ++k) {
            lo[k] = std::min(lo[k], pos[3 * (size_t)n + k]);
            hi[k] = std::max(hi[k], pos[3 * (size_t)n + k]);
        }
    double ext = std::max({hi[0] - lo[0], hi[1] - lo[1], hi[2] - lo[2], 1e-300});
    const double scale = 1023.0 / ext;
    std::vector<std::pair<uint32_t, int>> keys((size_t)E);
    for (int e = 0; e < E; ++e) {
        double c[3] = {0, 0, 0};
        for (int i = 0; i < 4; ++i)
            for (int k = 0; k < 3; ++k) c[k] += 0.25 * pos[3 * (size_t)tets[4 * (size_t)e + i] + k];
        uint32_t q[3];
        for (int k = 0; k < 3; ++k) {
            double t = (c[k] - lo[k]) * scale;
            q[k] = (uint32_t)std::min(1023.0, std::max(0.0, t));
        }
        keys[(size_t)e] = {spread10(q[0]) | (spread10(q[1]) << 1) | (spread10(q[2]) << 2), e};
    }
    std::sort(keys.begin(), keys.end());
    L.perm.resize((size_t)E);
    L.inv.resize((size_t)E);
    for (int s = 0; s < E; ++s) {
        L.perm[(size_t)s] = keys[(size_t)s].second;
        L.inv[(size_t)keys[(size_t)s].second] = s;
    }
    keys.clear();
    keys.shrink_to_fit();

    // 2. greedy patches of at most `pe` elements and `pn_max` distinct nodes.
    //    Every patch but the last has an even element count (pe is even), so
    //    each patch's per-element arrays start on a 16-byte boundary for the
    //    kernels' bulk copies; a patch closes only at an even count, keeping
    //    room for the four nodes of one more element under pn_max.
    std::vector<int> stamp((size_t)N, -1);
    L.elem_start.clear();
    L.elem_start.push_back(0);
    pe = pe & ~1;
    if (pe < 2) pe = 2;
    {
        int patch = 0, count = 0, nodes = 0;
        for (int s = 0; s < E; ++s) {
            const int32_t* t = &tets[4 * (size_t)L.perm[(size_t)s]];
            int fresh = 0;
            for (int i = 0; i < 4; ++i)
                if (stamp[(size_t)t[i]] != patch) fresh++;
            if (count > 0 && (count % 2) == 0 && (count + 1 > pe || nodes + fresh > pn_max - 4)) {
                L.elem_start.push_back(s);
                patch++;
                count = 0;
                nodes = 0;
                fresh = 4;
            }
            for (int i = 0; i < 4; ++i)
                if (stamp[(size_t)t[i]] != patch) {
                    stamp[(size_t)t[i]] = patch;
                    nodes++;
                }
            count++;
        }
        if (E > 0) L.elem_start.push_back(E);
    }
    const int P = (int)L.elem_start.size() - 1;

    // 3. local node lists (ascending global id) and element connectivity
    L.node_start.assign(1, 0);
    L.lnode_gid.clear();
    L.lconn.resize((size_t)E);
    std::vector<int> local((size_t)N, -1);
    std::vector<int> patch_count((size_t)N, 0);
    L.max_lnodes = 0;
    for (int p = 0; p < P; ++p) {
        std::vector<int> nodes;
        for (int s = L.elem_start[p]; s < L.elem_start[p + 1]; ++s) {
            const int32_t* t = &tets[4 * (size_t)L.perm[(size_t)s]];
            for (int i = 0; i < 4; ++i) nodes.push_back(t[i]);
        }
        std::sort(nodes.begin(), nodes.end());
        nodes.erase(std::unique(nodes.begin(), nodes.end()), nodes.end());
        for (size_t l = 0; l < nodes.size(); ++l) {
            local[(size_t)nodes[l]] = (int)l;
            patch_count[(size_t)nodes[l]]++;
        }
        for (int s = L.elem_start[p]; s < L.elem_start[p + 1]; ++s) {
            const int32_t* t = &tets[4 * (size_t)L.perm[(size_t)s]];
            L.lconn[(size_t)s] = make_ushort4((unsigned short)local[(size_t)t[0]], (unsigned short)local[(size_t)t[1]],
                                              (unsigned short)local[(size_t)t[2]], (unsigned short)local[(size_t)t[3]]);
        }
        L.lnode_gid.insert(L.lnode_gid.end(), nodes.begin(), nodes.end());
        L.node_start.push_back((int)L.lnode_gid.size());
        L.max_lnodes = std::max(L.max_lnodes, (int)nodes.size());
    }
    // nodes of no element (a MechanicalObject with unused points) go into
    // trailing patches without elements, at most max_lnodes each: the patch
    // kernels then form their mass rows (and CG directions) like any other
    // node's, with an empty stiffness sum
    if (P > 0) {
        std::vector<int> lone;
        for (int n = 0; n < N; ++n)
            if (patch_count[(size_t)n] == 0) lone.push_back(n);
        const size_t chunk = (size_t)std::max(L.max_lnodes, 1);
        for (size_t i = 0; i < lone.size(); i += chunk) {
            const size_t j = std::min(lone.size(), i + chunk);
            for (size_t k = i; k < j; ++k) patch_count[(size_t)lone[k]] = 1;
            L.lnode_gid.insert(L.lnode_gid.end(), lone.begin() + (long)i, lone.begin() + (long)j);
            L.node_start.push_back((int)L.lnode_gid.size());
            L.elem_start.push_back(E);
        }
    }
    const int P_all = (int)L.elem_start.size() - 1;

    // 4. boundary nodes: one partial slot per touching patch, in patch order;
    //    the first patch owns the node
    L.bnd_rowptr.assign((size_t)N + 1, 0);
    L.n_boundary = 0;
    for (int n = 0; n < N; ++n) {
        int c = patch_count[(size_t)n] > 1 ? patch_count[(size_t)n] : 0;
        L.bnd_rowptr[(size_t)n + 1] = L.bnd_rowptr[(size_t)n] + c;
        if (c) L.n_boundary++;
    }
    L.n_partials = L.bnd_rowptr[(size_t)N];
    std::vector<int> next(L.bnd_rowptr.begin(), L.bnd_rowptr.end() - 1);
    L.lnode_info.resize(L.lnode_gid.size());
    for (int p = 0; p < P_all; ++p)
        for (int l = L.node_start[p]; l < L.node_start[p + 1]; ++l) {
            const int g = L.lnode_gid[(size_t)l];
            if (patch_count[(size_t)g] <= 1) {
                L.lnode_info[(size_t)l] = -1;
            } else {
                const int slot = next[(size_t)g]++;
                L.lnode_info[(size_t)l] = 2 * slot + (slot == L.bnd_rowptr[(size_t)g] ? 1 : 0);
            }
        }

    // 5. per patch local CSR: local node -> (local element*4 + corner), sorted
    L.lrow.assign(L.lnode_gid.size() + 1, 0);
    for (int p = 0; p < P; ++p) {
        const int n0 = L.node_start[p];
        for (int s = L.elem_start[p]; s < L.elem_start[p + 1]; ++s) {
            const ushort4 c = L.lconn[(size_t)s];
            L.lrow[(size_t)n0 + c.x + 1]++;
            L.lrow[(size_t)n0 + c.y + 1]++;
            L.lrow[(size_t)n0 + c.z + 1]++;
            L.lrow[(size_t)n0 + c.w + 1]++;
        }
    }
    for (size_t l = 0; l < L.lnode_gid.size(); ++l) L.lrow[l + 1] += L.lrow[l];
    L.lslots.resize((size_t)E * 4);
    std::vector<int> fill(L.lrow.begin(), L.lrow.end() - 1);
    for (int p = 0; p < P; ++p) {
        const int n0 = L.node_start[p], s0 = L.elem_start[p];
        for (int s = s0; s < L.elem_start[p + 1]; ++s) {
            const ushort4 c = L.lconn[(size_t)s];
            const unsigned short ln[4] = {c.x, c.y, c.z, c.w};
            for (int i = 0; i < 4; ++i)
                L.lslots[(size_t)fill[(size_t)n0 + ln[i]]++] = (uint16_t)((s - s0) * 4 + i);
        }
    }

}

// Node -> (storage position*4 + corner) table with each row sorted by the
// ORIGINAL element index, so a node sums its terms in the reference's
// element-loop order whatever the storage order.
void build_node_csr(int N, int E, const int32_t* tets, const std::vector<int>& inv, std::vector<int>& rowptr,
                    std::vector<int>& slots, int& max_valence)
{
    rowptr.assign((size_t)N + 1, 0);
    for (size_t i = 0; i < (size_t)E * 4; ++i) rowptr[(size_t)tets[i] + 1]++;
    max_valence = 0;
    for (int n = 0; n < N; ++n) {
        max_valence = std::max(max_valence, rowptr[(size_t)n + 1]);
        rowptr[(size_t)n + 1] += rowptr[(size_t)n];
    }
    slots.resize((size_t)E * 4);
    std::vector<int> pos(rowptr.begin(), rowptr.end() - 1);
    for (int e = 0; e < E; ++e)
        for (int c = 0; c < 4; ++c)
            slots[(size_t)pos[(size_t)tets[4 * (size_t)e + c]]++] = inv[(size_t)e] * 4 + c;
}

}  // namespace sgb
