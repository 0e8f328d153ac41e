// Instantiates tfem_impl.cuh for one real type and exports its table.
// Expects SGB_NS, SGB_REAL and SGB_TABLE to be defined.
#include "tfem_impl.cuh"
#if SGB_USES_PATCHES
#include "batch_impl.cuh"
#endif
#include "variants.h"

namespace SGB_NS {
static void v_init(TfemMesh* m, const double* y, int ny, const double* p, int np, const double* l, int nl,
                   double* vol, cudaStream_t s)
{
    launch_init<SGB_REAL>(m, y, ny, p, np, l, nl, vol, s);
}
static void v_add_force(TfemMesh* m, const double* x, void* f, cudaStream_t s)
{
    api_add_force<SGB_REAL, SGB_REAL>(m, x, (SGB_REAL*)f, s);
}
static void v_add_dforce(TfemMesh* m, const void* dx, void* df, double k, cudaStream_t s)
{
    api_add_dforce<SGB_REAL>(m, (const SGB_REAL*)dx, (SGB_REAL*)df, (SGB_REAL)k, s);
}
static void v_scene_step(Scene* sc, double* terms, int mass_first, cudaStream_t s)
{
    // FP32 runs the fused patch matvec (CG and PCG); FP64 (FMA) is bound by
    // the FP64 issue rate, where the element-order path with its plain gather
    // is faster
    if (SGB_USES_PATCHES && sizeof(SGB_REAL) == 4 && sc->mesh->pl.n_patches > 0 &&
        sc->mesh->method != METHOD_SMALL) {
        if (sc->replace_every > 0 && sc->shadow && sc->shadow->pl.n_patches > 0)
            scene_step_refined<SGB_REAL>(sc, mass_first, s);
        else
            scene_step_patch<SGB_REAL>(sc, mass_first, s);
    }
    else
        scene_step<SGB_REAL>(sc, terms, mass_first, s);
}
static int v_prepare(TfemMesh* m) { return m->pl.n_patches > 0 ? prepare_patch<SGB_REAL>(m) : 0; }
#if SGB_USES_PATCHES
static int v_batch_prepare(int pe, int* grid_patch)
{
    return batch_prepare<SGB_REAL>(pe, grid_patch);
}
static void v_batch_record(const BatchLaunch& b, cudaStream_t s) { batch_record_step<SGB_REAL>(b, s); }
#else
static int (*const v_batch_prepare)(int, int*) = nullptr;
static void (*const v_batch_record)(const BatchLaunch&, cudaStream_t) = nullptr;
#endif
static void v_stiffness_blocks(TfemMesh* m, const int* cptr, const int* contrib, int n_blocks, double* out,
                               cudaStream_t s)
{
    launch_stiffness_blocks<SGB_REAL>(m, cptr, contrib, n_blocks, out, s);
}
static void v_plastic_scale(TfemMesh* m, const double* y, int ny, const double* p, int np, const double* l, int nl,
                            cudaStream_t s)
{
    launch_plastic_scale<SGB_REAL>(m, y, ny, p, np, l, nl, s);
}
}  // namespace SGB_NS

namespace sgb {
const VariantOps SGB_TABLE = {SGB_VARIANT_NAME,     sizeof(SGB_REAL),     SGB_USES_PATCHES,
                              SGB_NS::v_init,       SGB_NS::v_add_force,  SGB_NS::v_add_dforce,
                              SGB_NS::v_scene_step, SGB_NS::v_prepare,   SGB_NS::v_batch_prepare,
                              SGB_NS::v_batch_record, SGB_NS::v_stiffness_blocks, SGB_NS::v_plastic_scale};
}
