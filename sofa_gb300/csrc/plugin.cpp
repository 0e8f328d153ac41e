// C ABI of the component layer (include/sofa_gb300_scene.h): scene files and
// the plugin entry points PluginManager looks up.
#include <cstring>
#include <string>

#include "../../include/sofa_gb300_scene.h"
#include "scene_graph.h"

namespace sgb {
void set_last_error(const std::string& msg);  // capi.cu: the message sgb_last_error() returns
}

struct sgb_sofa_scene {
    sgb::scn::Scene scene;
};

namespace {

int fail(int rc, const std::string& m)
{
    sgb::set_last_error(m);
    return rc;
}

bool g_initialized = false;

std::string component_list()
{
    std::string s;
    for (const std::string& c : sgb::scn::default_factory().class_names()) {
        if (!s.empty()) s += ' ';
        s += c;
    }
    return s;
}

}  // namespace

extern "C" {

int sgb_sofa_scene_load(sgb_sofa_scene_t** out, const char* xml_text, int precision)
{
    if (!out || !xml_text) return fail(SGB_ERR_INVALID_ARGUMENT, "sgb_sofa_scene_load: NULL argument");
    *out = nullptr;
    if (precision < -1 || precision > SGB_PRECISION_FP64_FMA)
        return fail(SGB_ERR_INVALID_ARGUMENT, "sgb_sofa_scene_load: unknown precision");
    auto* h = new (std::nothrow) sgb_sofa_scene();
    if (!h) return fail(SGB_ERR_OUT_OF_MEMORY, "sgb_sofa_scene_load: out of host memory");
    h->scene.precision_override = precision;
    std::string err;
    int rc = sgb::scn::parse_scene_xml(xml_text, sgb::scn::default_factory(), h->scene, &err);
    if (!rc) rc = h->scene.init_host(&err);
    if (rc) {
        delete h;
        return fail(rc, err);
    }
    *out = h;
    return SGB_OK;
}

int sgb_sofa_scene_destroy(sgb_sofa_scene_t* scene)
{
    delete scene;
    return SGB_OK;
}

int sgb_sofa_scene_describe(const sgb_sofa_scene_t* scene, char* buf, size_t buf_size, size_t* needed)
{
    if (!scene) return fail(SGB_ERR_INVALID_ARGUMENT, "sgb_sofa_scene_describe: NULL scene");
    const std::string d = scene->scene.describe();
    if (needed) *needed = d.size() + 1;
    if (buf && buf_size > 0) {
        const size_t n = d.size() < buf_size - 1 ? d.size() : buf_size - 1;
        std::memcpy(buf, d.data(), n);
        buf[n] = '\0';
    }
    return SGB_OK;
}

int sgb_sofa_scene_bodies(const sgb_sofa_scene_t* scene, int* n_bodies)
{
    if (!scene || !n_bodies) return fail(SGB_ERR_INVALID_ARGUMENT, "sgb_sofa_scene_bodies: NULL argument");
    *n_bodies = (int)scene->scene.bodies.size();
    return SGB_OK;
}

int sgb_sofa_scene_body_info(const sgb_sofa_scene_t* scene, int body, int* n_nodes, int* n_tets, int* method,
                             int* precision, int* n_fixed)
{
    if (!scene || body < 0 || body >= (int)scene->scene.bodies.size())
        return fail(SGB_ERR_NOT_FOUND, "sgb_sofa_scene_body_info: no such body");
    const sgb::scn::Body& b = scene->scene.bodies[(size_t)body];
    if (n_nodes) *n_nodes = (int)(b.rest.size() / 3);
    if (n_tets) *n_tets = (int)(b.tets.size() / 4);
    if (method) *method = b.method;
    if (precision) *precision = b.precision;
    if (n_fixed) *n_fixed = b.params.fix_all ? (int)(b.rest.size() / 3) : (int)b.fixed.size();
    return SGB_OK;
}

int sgb_sofa_scene_body_solver(const sgb_sofa_scene_t* scene, int body, int* linear_solver, int* preconditioner,
                               int* preconditioner_rate, int* iterations, double* tolerance)
{
    if (!scene || body < 0 || body >= (int)scene->scene.bodies.size())
        return fail(SGB_ERR_NOT_FOUND, "sgb_sofa_scene_body_solver: no such body");
    const sgb_scene_params& p = scene->scene.bodies[(size_t)body].params;
    if (linear_solver) *linear_solver = p.linear_solver;
    if (preconditioner) *preconditioner = p.preconditioner;
    if (preconditioner_rate) *preconditioner_rate = p.preconditioner_rate > 1 ? p.preconditioner_rate : 1;
    if (iterations) *iterations = p.cg_iterations;
    if (tolerance) *tolerance = p.cg_tolerance;
    return SGB_OK;
}

int sgb_sofa_scene_body_arrays(const sgb_sofa_scene_t* scene, int body, int32_t* tetrahedra, double* node_masses,
                               int32_t* fixed)
{
    if (!scene || body < 0 || body >= (int)scene->scene.bodies.size())
        return fail(SGB_ERR_NOT_FOUND, "sgb_sofa_scene_body_arrays: no such body");
    const sgb::scn::Body& b = scene->scene.bodies[(size_t)body];
    const size_t N = b.rest.size() / 3;
    if (tetrahedra) std::memcpy(tetrahedra, b.tets.data(), sizeof(int32_t) * b.tets.size());
    if (node_masses) {
        if (b.node_masses.size() == N)
            std::memcpy(node_masses, b.node_masses.data(), sizeof(double) * N);
        else
            for (size_t i = 0; i < N; ++i) node_masses[i] = b.params.vertex_mass;
    }
    if (fixed) {
        if (b.params.fix_all)
            for (size_t i = 0; i < N; ++i) fixed[i] = (int32_t)i;
        else
            std::memcpy(fixed, b.fixed.data(), sizeof(int32_t) * b.fixed.size());
    }
    return SGB_OK;
}

int sgb_sofa_scene_init_device(sgb_sofa_scene_t* scene)
{
    if (!scene) return fail(SGB_ERR_INVALID_ARGUMENT, "sgb_sofa_scene_init_device: NULL scene");
    std::string err;
    int rc = scene->scene.init_device(&err);
    return rc ? fail(rc, err) : SGB_OK;
}

int sgb_sofa_scene_animate(sgb_sofa_scene_t* scene, int n_steps)
{
    if (!scene || n_steps < 0) return fail(SGB_ERR_INVALID_ARGUMENT, "sgb_sofa_scene_animate: invalid argument");
    std::string err;
    int rc = scene->scene.animate(n_steps, &err);
    return rc ? fail(rc, err) : SGB_OK;
}

int sgb_sofa_scene_reset(sgb_sofa_scene_t* scene)
{
    if (!scene) return fail(SGB_ERR_INVALID_ARGUMENT, "sgb_sofa_scene_reset: NULL scene");
    std::string err;
    int rc = scene->scene.reset(&err);
    return rc ? fail(rc, err) : SGB_OK;
}

int sgb_sofa_scene_unload(sgb_sofa_scene_t* scene)
{
    if (!scene) return fail(SGB_ERR_INVALID_ARGUMENT, "sgb_sofa_scene_unload: NULL scene");
    return scene->scene.unload();
}

int sgb_sofa_scene_get_positions(sgb_sofa_scene_t* scene, int body, double* x_host)
{
    if (!scene || !x_host || body < 0 || body >= (int)scene->scene.bodies.size())
        return fail(SGB_ERR_NOT_FOUND, "sgb_sofa_scene_get_positions: no such body");
    sgb::scn::Body& b = scene->scene.bodies[(size_t)body];
    if (b.scene) return sgb_scene_get_state(b.scene, x_host, nullptr);
    const std::vector<double>* x = &b.rest;
    for (auto& o : b.node->objects)
        if (o->class_name() == "MechanicalObject") {
            auto it = o->out_reals.find("position");
            if (it != o->out_reals.end() && it->second.size() == b.rest.size()) x = &it->second;
            break;
        }
    std::memcpy(x_host, x->data(), sizeof(double) * x->size());
    return SGB_OK;
}

int sgb_sofa_scene_get_von_mises(sgb_sofa_scene_t* scene, int body, double* per_element_host,
                                 double* per_node_host)
{
    if (!scene || !per_element_host || body < 0 || body >= (int)scene->scene.bodies.size())
        return fail(SGB_ERR_NOT_FOUND, "sgb_sofa_scene_get_von_mises: no such body");
    sgb::scn::Body& b = scene->scene.bodies[(size_t)body];
    if (b.von_mises_mode == 0)
        return fail(SGB_ERR_INVALID_ARGUMENT, "sgb_sofa_scene_get_von_mises: computeVonMisesStress is 0");
    if (!b.scene)
        return fail(SGB_ERR_INVALID_ARGUMENT, "sgb_sofa_scene_get_von_mises: the device is not initialised yet");
    return sgb_scene_von_mises(b.scene, b.von_mises_mode, per_element_host, per_node_host);
}

int sgb_sofa_scene_get_residual(sgb_sofa_scene_t* scene, int body, double* residual)
{
    if (!scene || !residual || body < 0 || body >= (int)scene->scene.bodies.size())
        return fail(SGB_ERR_NOT_FOUND, "sgb_sofa_scene_get_residual: no such body");
    sgb::scn::Body& b = scene->scene.bodies[(size_t)body];
    if (!b.params.compute_residual)
        return fail(SGB_ERR_INVALID_ARGUMENT, "sgb_sofa_scene_get_residual: computeResidual is 0");
    if (!b.scene)
        return fail(SGB_ERR_INVALID_ARGUMENT, "sgb_sofa_scene_get_residual: the device is not initialised yet");
    return sgb_scene_residual(b.scene, residual);
}

int sgb_sofa_scene_time(const sgb_sofa_scene_t* scene, double* t)
{
    if (!scene || !t) return fail(SGB_ERR_INVALID_ARGUMENT, "sgb_sofa_scene_time: NULL argument");
    *t = scene->scene.time;
    return SGB_OK;
}

void* sgb_object_factory_new(void) { return new (std::nothrow) sgb::scn::ObjectFactory(); }

void sgb_object_factory_delete(void* factory) { delete static_cast<sgb::scn::ObjectFactory*>(factory); }

int sgb_object_factory_has(const void* factory, const char* class_name)
{
    if (!factory || !class_name) return 0;
    return static_cast<const sgb::scn::ObjectFactory*>(factory)->has(class_name) ? 1 : 0;
}

int sgb_object_factory_count(const void* factory)
{
    if (!factory) return 0;
    return (int)static_cast<const sgb::scn::ObjectFactory*>(factory)->class_names().size();
}

void initExternalModule(void)
{
    if (g_initialized) return;
    (void)sgb::scn::default_factory();
    g_initialized = true;
}

const char* getModuleName(void) { return "SofaGB300"; }

const char* getModuleVersion(void) { return "0.1"; }

const char* getModuleLicense(void) { return "LGPL"; }

const char* getModuleDescription(void)
{
    return "GB300 (sm_103a) implicit corotational tetrahedral FEM: TetrahedronFEMForceField, EulerImplicitSolver, "
           "CGLinearSolver, UniformMass/DiagonalMass, FixedProjectiveConstraint";
}

const char* getModuleComponentList(void)
{
    static const std::string list = component_list();
    return list.c_str();
}

bool moduleIsInitialized(void) { return g_initialized; }

void registerObjects(void* factory)
{
    if (factory) sgb::scn::register_components(*static_cast<sgb::scn::ObjectFactory*>(factory));
}

}  // extern "C"
