// Function table of one precision variant of the kernels (tfem_impl.cuh).
#pragma once
#include <cuda_runtime.h>

#include "sgb_internal.h"

namespace sgb {

struct VariantOps {
    const char* name;
    size_t real_size;
    int uses_patches;  // fused patch matvec (the reference-rounding variant keeps the element-order gather)
    void (*init)(TfemMesh*, const double* young, int ny, const double* poisson, int np, const double* lsf, int nl,
                 double* vol, cudaStream_t);
    void (*add_force)(TfemMesh*, const double* x, void* f, cudaStream_t);
    void (*add_dforce)(TfemMesh*, const void* dx, void* df, double kfactor, cudaStream_t);
    void (*scene_step)(Scene*, double* dot_terms, int mass_first, cudaStream_t);
    int (*prepare)(TfemMesh*);  // kernel attributes; returns the patch-kernel grid
    // batch engine (null for the reference-rounding variant)
    int (*batch_prepare)(int pe, int* grid_patch);  // returns the SM count, -1 on failure
    void (*batch_record)(const BatchLaunch&, cudaStream_t);
    // assembled stiffness blocks (BSR, 3x3) at the current rotations
    void (*stiffness_blocks)(TfemMesh*, const int* cptr, const int* contrib, int n_blocks, double* out,
                             cudaStream_t);
    // mixed plasticity: per-element scale of the stored strain (plastic_scale)
    void (*plastic_scale)(TfemMesh*, const double* young, int ny, const double* poisson, int np, const double* lsf,
                          int nl, cudaStream_t);
};

extern const VariantOps ops_fp64_exact;
extern const VariantOps ops_fp64_fast;
extern const VariantOps ops_mixed;

const VariantOps* variant_for(int precision);

}  // namespace sgb
