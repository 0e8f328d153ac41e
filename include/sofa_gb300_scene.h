/* SOFA scene files and plugin entry points of libsofa_gb300.
 *
 * Component layer above the C ABI of sofa_gb300.h: a scene written for the
 * reference (.scn XML with RegularGridTopology, Hexa2TetraTopologicalMapping,
 * TetrahedronSetTopologyContainer, MechanicalObject, BoxROI,
 * FixedProjectiveConstraint, UniformMass / DiagonalMass,
 * TetrahedronFEMForceField, EulerImplicitSolver, CGLinearSolver) is parsed
 * into a graph of components with the reference's class and Data names, and
 * every node that holds an EulerImplicitSolver becomes one GPU scene.
 * Visual, collision-pipeline and plugin-declaration components are accepted
 * and listed as ignored; an unknown component is an error
 * (SGB_ERR_NOT_SUPPORTED), as the reference's ObjectFactory refuses a class
 * it does not know.
 *
 * Functions return SGB_OK or a negative SGB_ERR_* code; sgb_last_error()
 * holds the message.
 */
#ifndef SOFA_GB300_SCENE_H
#define SOFA_GB300_SCENE_H

#include <stdbool.h>
#include <stddef.h>

#include "sofa_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct sgb_sofa_scene sgb_sofa_scene_t;

/* Parses the XML text of a scene and initialises it on the host: topology,
 * positions, masses, fixed indices, solver parameters (the init pass of
 * sofa::simulation::node::initRoot). No device memory is used.
 * precision: SGB_PRECISION_* to force one, or -1 to follow each
 * MechanicalObject's template (Vec3f / CudaVec3f -> SGB_PRECISION_MIXED,
 * Vec3d / Vec3 / CudaVec3d -> SGB_PRECISION_FP64). */
int sgb_sofa_scene_load(sgb_sofa_scene_t** out, const char* xml_text, int precision);
int sgb_sofa_scene_destroy(sgb_sofa_scene_t* scene);

/* JSON description of the parsed scene: bodies with their sizes and solver
 * parameters, the node tree with every component and the Data it sets,
 * ignored components and warnings. Writes at most buf_size bytes
 * (NUL-terminated when buf_size > 0); *needed = length + 1. */
int sgb_sofa_scene_describe(const sgb_sofa_scene_t* scene, char* buf, size_t buf_size, size_t* needed);

/* Number of simulated bodies and the sizes of one of them. */
int sgb_sofa_scene_bodies(const sgb_sofa_scene_t* scene, int* n_bodies);
int sgb_sofa_scene_body_info(const sgb_sofa_scene_t* scene, int body, int* n_nodes, int* n_tets, int* method,
                             int* precision, int* n_fixed);

/* Linear solver of a body as assembled from the scene: SGB_SOLVER_CG or
 * SGB_SOLVER_PCG, its preconditioner (SGB_PRECOND_*) and assembling rate,
 * iterations and tolerance. Any output may be NULL. */
int sgb_sofa_scene_body_solver(const sgb_sofa_scene_t* scene, int body, int* linear_solver, int* preconditioner,
                               int* preconditioner_rate, int* iterations, double* tolerance);

/* Host arrays of a body as assembled from the scene: tetrahedra (n_tets x 4),
 * lumped node masses (n_nodes; all equal to the vertex mass for a
 * UniformMass) and fixed indices (n_fixed). NULL pointers are skipped. */
int sgb_sofa_scene_body_arrays(const sgb_sofa_scene_t* scene, int body, int32_t* tetrahedra, double* node_masses,
                               int32_t* fixed);

/* Creates the GPU objects of every body (sgb_tfem_create + sgb_scene_create). */
int sgb_sofa_scene_init_device(sgb_sofa_scene_t* scene);

/* DefaultAnimationLoop::step, n_steps times, on every body
 * (DefaultAnimationLoop.cpp:273-325). Initialises the device first if
 * needed. Stream-ordered; sgb_sofa_scene_get_positions synchronises. */
int sgb_sofa_scene_animate(sgb_sofa_scene_t* scene, int n_steps);

/* SofaPhysicsAPI::reset (applications/projects/SofaPhysicsAPI/src/
 * SofaPhysicsAPI/SofaPhysicsAPI.h:98-99; sofa::simulation::node::reset):
 * every body's positions back to their initial values and velocities to
 * their initial values (zero unless the scene set them), as
 * MechanicalObject::reset does (Sofa/Component/StateContainer/src/sofa/
 * component/statecontainer/MechanicalObject.inl:1204-1225); plastic strains
 * cleared (TetrahedronFEMForceField.inl:1382-1388); WriteState rewound; time
 * 0. The solvers keep their own state (the reference's CGLinearSolver has no
 * reset). Device objects are kept; synchronous. */
int sgb_sofa_scene_reset(sgb_sofa_scene_t* scene);

/* SofaPhysicsAPI::unload (SofaPhysicsAPI.h:74-75) for the device: releases
 * every body's GPU objects (device memory) and keeps the parsed scene; the
 * next sgb_sofa_scene_animate (or init_device) creates them again and starts
 * from the initial state. Destroy the scene itself with
 * sgb_sofa_scene_destroy. */
int sgb_sofa_scene_unload(sgb_sofa_scene_t* scene);

/* Positions of a body (n_nodes x 3 doubles): the current state once the
 * device is initialised, else the initial positions. */
int sgb_sofa_scene_get_positions(sgb_sofa_scene_t* scene, int body, double* x_host);

/* vonMisesPerElement / vonMisesPerNode of a body whose
 * TetrahedronFEMForceField sets computeVonMisesStress (1 or 2), at its
 * current state (TetrahedronFEMForceField.inl:2197-2374); per_node_host may be
 * NULL. SGB_ERR_INVALID_ARGUMENT when the force field does not compute it or
 * the device is not initialised yet. Synchronous. */
int sgb_sofa_scene_get_von_mises(sgb_sofa_scene_t* scene, int body, double* per_element_host,
                                 double* per_node_host);

/* The Data `residual` of a body's EulerImplicitSolver with computeResidual
 * set (EulerImplicitSolver.cpp:48-49, 314-338): r.r of the last step's
 * residual. SGB_ERR_INVALID_ARGUMENT when computeResidual is 0 or the device
 * is not initialised yet. Synchronous. */
int sgb_sofa_scene_get_residual(sgb_sofa_scene_t* scene, int body, double* residual);

/* Simulated time (steps x dt). */
int sgb_sofa_scene_time(const sgb_sofa_scene_t* scene, double* t);

/* The object factory the components are registered in, for a host that
 * loads this library as a plugin: sgb_object_factory_new creates an empty
 * factory, registerObjects(factory) fills it, the queries read it. */
void* sgb_object_factory_new(void);
void sgb_object_factory_delete(void* factory);
int sgb_object_factory_has(const void* factory, const char* class_name);
int sgb_object_factory_count(const void* factory);

/* Plugin entry points looked up by PluginManager::loadPlugin with dlsym
 * (Sofa/framework/Helper/src/sofa/helper/system/PluginManager.cpp:88-94,
 * 229-260; SofaCUDA's init.cpp:33-59): initExternalModule and getModuleName
 * are required, the others optional. registerObjects takes the host's
 * factory; here that is a factory from sgb_object_factory_new, which has the
 * registration shape of sofa::core::ObjectFactory (class name, description,
 * module, creator). */
void initExternalModule(void);
const char* getModuleName(void);
const char* getModuleVersion(void);
const char* getModuleLicense(void);
const char* getModuleDescription(void);
const char* getModuleComponentList(void);
bool moduleIsInitialized(void);
void registerObjects(void* factory);

#ifdef __cplusplus
}
#endif

#endif
