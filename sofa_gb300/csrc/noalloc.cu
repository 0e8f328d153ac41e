// addDForce for callers that cannot allocate device memory.
//
// Some callers cannot call cudaMalloc or cudaFree at the point where they
// need a force derivative: a host framework that hands out device buffers
// from its own pool (SOFA's vector_device-style mirrors), a real-time loop
// that must not hit the implicit device synchronisation cudaMalloc/cudaFree
// cause, or code that runs where the runtime forbids new allocations. The
// handle-based entry points allocate their buffers in sgb_tfem_create; this
// one takes every input and output from the caller and keeps its only
// scratch -- the four corner terms of each tetrahedron between the element
// pass and the node gather -- in a fixed array in the library's own device
// memory, so a call allocates nothing.
//
// The array holds kNoAllocMaxTets tetrahedra (12 floats each, 12 MiB) and
// every GPU that loads the library keeps it until the process exits. All
// calls share it and it keeps the previous call's contents; nothing in it
// has to start at zero, because the element pass overwrites every entry the
// gather then reads. Two calls that overlap on the GPU (different streams,
// no ordering between them) race on the array and give wrong results.
// The array's device address is looked up once per device and kept; a
// cudaDeviceReset (or any teardown of the primary context) in the same
// process reloads the module and may move the array, so this entry point
// is not to be called again after one.
//
// Node and slot indices come from the caller. The kernels check them
// against n_nodes and 4*n_tets before any access: an out-of-range entry is
// skipped (it contributes nothing), so a bad table gives a wrong df but
// never an access outside the caller's arrays or the scratch.
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>
#include <string>

#include "../../include/sofa_gb300.h"
#include "tfem_math.cuh"

namespace {

constexpr int kNoAllocMaxTets = 1 << 18;  // 262,144 tetrahedra
constexpr int kMaxDevices = 64;

static __device__ __align__(256) float g_noalloc_corner_terms[12 * kNoAllocMaxTets];

std::mutex g_setup_mutex;
void* g_scratch_addr[kMaxDevices] = {nullptr};
int g_sm_count[kMaxDevices] = {0};


// Once per device, with that device current: the device address of the
// array. In host code the array's name is only a host-side stand-in, so the
// kernels receive this address instead.
cudaError_t scratch_for_current_device(float** out, int* sm_count)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_addr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_corner_terms);
        if (e != cudaSuccess) return e;
        int sms = 0;
        e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (e != cudaSuccess) return e;
        g_sm_count[dev] = sms > 0 ? sms : 1;
        g_scratch_addr[dev] = p;
    }
    *out = (float*)g_scratch_addr[dev];
    *sm_count = g_sm_count[dev];
    return cudaSuccess;
}

// Element pass: corner terms R K (R^T dx) kfactor of the corotational
// stiffness (applyStiffnessCorotational, TetrahedronFEMForceField.inl:1193-1237).
__global__ void __launch_bounds__(128) k_noalloc_elements(int n_nodes, int n_tets, const int4* __restrict__ tets,
                                                          const float* __restrict__ rot,
                                                          const float* __restrict__ K,
                                                          const float* __restrict__ J,
                                                          const float* __restrict__ dx, float kfactor,
                                                          float* __restrict__ scratch)
{
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n_tets) return;
    const size_t En = (size_t)n_tets;
    const int4 t = tets[e];
    const int node[4] = {t.x, t.y, t.z, t.w};
    // a node index outside [0, n_nodes) reads nothing: its values count as zero
    bool ok[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) ok[i] = (unsigned)node[i] < (unsigned)n_nodes;
    float Rm[9], Ke[3], Je[12], X[12], F[12];
#pragma unroll
    for (int i = 0; i < 9; ++i) Rm[i] = rot[i * En + e];
#pragma unroll
    for (int i = 0; i < 3; ++i) Ke[i] = K[i * En + e];
#pragma unroll
    for (int i = 0; i < 12; ++i) Je[i] = J[i * En + e];
    float d[4][3];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int k = 0; k < 3; ++k) d[i][k] = ok[i] ? dx[3 * (size_t)node[i] + k] : 0.f;
    // values relative to node a: J^T annihilates translations
#pragma unroll
    for (int i = 3; i >= 0; --i)
#pragma unroll
        for (int k = 0; k < 3; ++k) d[i][k] -= d[0][k];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int k = 0; k < 3; ++k)
            X[3 * i + k] = Rm[3 * k] * d[i][0] + Rm[3 * k + 1] * d[i][1] + Rm[3 * k + 2] * d[i][2];
    sgb::element_force(F, X, Ke, Je, kfactor);
    float* o = scratch + 12 * (size_t)e;
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int k = 0; k < 3; ++k) o[3 * i + k] = Rm[k] * F[3 * i] + Rm[3 + k] * F[3 * i + 1] + Rm[6 + k] * F[3 * i + 2];
}

// Node gather: each node subtracts its (tetrahedron, corner) terms in slot
// order, no atomics.
__global__ void __launch_bounds__(256) k_noalloc_gather(int n_nodes, int n_slots, const int* __restrict__ rowptr,
                                                        const int* __restrict__ slots,
                                                        const float* __restrict__ scratch, float* __restrict__ df)
{
    for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < n_nodes; n += gridDim.x * blockDim.x) {
        float a0 = df[3 * (size_t)n], a1 = df[3 * (size_t)n + 1], a2 = df[3 * (size_t)n + 2];
        // row bounds outside [0, n_slots] and slots outside [0, 4 n_tets) are skipped
        const int s0 = max(rowptr[n], 0), s1 = min(rowptr[n + 1], n_slots);
        for (int s = s0; s < s1; ++s) {
            const int slot = slots[s];
            if ((unsigned)slot >= (unsigned)n_slots) continue;
            const float* c = scratch + 3 * (size_t)slot;
            a0 -= c[0];
            a1 -= c[1];
            a2 -= c[2];
        }
        df[3 * (size_t)n] = a0;
        df[3 * (size_t)n + 1] = a1;
        df[3 * (size_t)n + 2] = a2;
    }
}

}  // namespace

namespace sgb {
void set_last_error(const std::string& msg);  // capi.cu: the message sgb_last_error() returns
}

extern "C" int sgb_tfem_add_dforce_f32_noalloc(int n_nodes, int n_tets, const int32_t* tetrahedra_dev,
                                               const float* rotations_dev, const float* stiffness_dev,
                                               const float* strain_displacement_dev, const int32_t* node_rowptr_dev,
                                               const int32_t* node_slots_dev, const float* dx_dev, float* df_dev,
                                               float kfactor, void* stream)
{
    if (n_nodes <= 0 || n_tets < 0) {
        sgb::set_last_error("sgb_tfem_add_dforce_f32_noalloc: n_nodes must be positive and n_tets non-negative");
        return SGB_ERR_INVALID_ARGUMENT;
    }
    if (n_tets > kNoAllocMaxTets) {
        sgb::set_last_error("sgb_tfem_add_dforce_f32_noalloc: " + std::to_string(n_tets) +
                          " tetrahedra exceed the fixed scratch of " + std::to_string(kNoAllocMaxTets) +
                          " tetrahedra; use sgb_tfem_add_dforce_f32 on a handle for larger meshes");
        return SGB_ERR_INVALID_ARGUMENT;
    }
    if (!node_rowptr_dev || !dx_dev || !df_dev ||
        (n_tets > 0 && (!tetrahedra_dev || !rotations_dev || !stiffness_dev || !strain_displacement_dev ||
                        !node_slots_dev))) {
        sgb::set_last_error("sgb_tfem_add_dforce_f32_noalloc: NULL array");
        return SGB_ERR_INVALID_ARGUMENT;
    }
    if (n_tets > 0 && ((uintptr_t)tetrahedra_dev & 15u) != 0) {
        sgb::set_last_error("sgb_tfem_add_dforce_f32_noalloc: tetrahedra_dev must be 16-byte aligned");
        return SGB_ERR_INVALID_ARGUMENT;
    }
    if (n_tets == 0) return SGB_OK;
    float* scratch = nullptr;
    int sms = 1;
    cudaError_t e = scratch_for_current_device(&scratch, &sms);
    if (e != cudaSuccess) {
        sgb::set_last_error(std::string("sgb_tfem_add_dforce_f32_noalloc: scratch set-up: ") + cudaGetErrorString(e));
        return SGB_ERR_CUDA;
    }
    cudaStream_t s = (cudaStream_t)stream;
    k_noalloc_elements<<<(n_tets + 127) / 128, 128, 0, s>>>(n_nodes, n_tets, (const int4*)tetrahedra_dev, rotations_dev,
                                                           stiffness_dev, strain_displacement_dev, dx_dev, kfactor,
                                                           scratch);
    // grid-stride gather: at most 8 resident 256-thread CTAs per SM
    int grid = (n_nodes + 255) / 256;
    if (grid > sms * 8) grid = sms * 8;
    k_noalloc_gather<<<grid, 256, 0, s>>>(n_nodes, 4 * n_tets, node_rowptr_dev, node_slots_dev, scratch, df_dev);
    e = cudaGetLastError();
    if (e != cudaSuccess) {
        sgb::set_last_error(std::string("sgb_tfem_add_dforce_f32_noalloc: launch: ") + cudaGetErrorString(e));
        return SGB_ERR_CUDA;
    }
    return SGB_OK;
}

