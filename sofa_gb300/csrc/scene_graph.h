// Component layer: a scene graph of SOFA-named components (Node, objects with
// named Data fields, an object factory) that maps the reference's soft-body
// scenes onto the library's scenes. It mirrors the shapes of
// sofa::simulation::Node, sofa::core::objectmodel::BaseObject / Data and
// sofa::core::ObjectFactory (Sofa/framework/Core/src/sofa/core/ObjectFactory.h)
// for the component subset of the implicit tetrahedral-FEM step; it is not
// linked against SOFA. Host code only; the device work goes through the
// C ABI of sofa_gb300.h.
#pragma once
#include <functional>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "../../include/sofa_gb300.h"

namespace sgb {
namespace scn {

class Node;
class Scene;

// One Data field: its name, help text, textual value (as written in the
// scene or the default) and whether the scene set it. A value starting with
// '@' is a link to another component's Data ("@../grid.position") or to a
// component ("@topo").
struct DataField {
    std::string name;
    std::string value;
    std::string help;
    bool is_set = false;
};

class BaseObject {
public:
    explicit BaseObject(std::string cls) : class_name_(std::move(cls)) {}
    virtual ~BaseObject() = default;

    const std::string& class_name() const { return class_name_; }
    std::string name;
    std::string template_name;
    Node* context = nullptr;

    // Data declaration and access (declaration order is kept for listings)
    void declare(const std::string& n, const std::string& def, const std::string& help);
    bool has_data(const std::string& n) const;
    DataField* data(const std::string& n);
    const DataField* data(const std::string& n) const;
    const std::vector<DataField>& fields() const { return fields_; }
    // sets a Data from the scene; returns false for an unknown attribute
    bool set(const std::string& n, const std::string& v);
    bool is_set(const std::string& n) const;

    // typed reads of a Data, following links to other components' Data
    std::vector<double> get_reals(Scene& s, const std::string& n);
    std::vector<int> get_ints(Scene& s, const std::string& n);
    double get_real(Scene& s, const std::string& n);
    int get_int(Scene& s, const std::string& n);
    bool get_bool(Scene& s, const std::string& n);
    std::string get_string(const std::string& n) const;

    // values computed by init (RegularGridTopology.position, BoxROI.indices, ...)
    std::map<std::string, std::vector<double>> out_reals;
    std::map<std::string, std::vector<int>> out_ints;

    // host-side initialisation (topology, masses, index sets); called once,
    // in dependency order, by Scene::init
    virtual void init(Scene&) {}
    bool initialized = false;
    bool initializing = false;
    // true for components that have no effect on the mechanical step
    // (visual, collision pipeline, plugin declarations)
    virtual bool ignored() const { return false; }
    // true for components that keep attributes they do not declare (drawing
    // options and other Data with no effect on the step) without a warning
    virtual bool permissive() const { return false; }

private:
    std::string class_name_;
    std::vector<DataField> fields_;
};

class Node {
public:
    std::string name;
    Node* parent = nullptr;
    std::vector<std::unique_ptr<BaseObject>> objects;
    std::vector<std::unique_ptr<Node>> children;
    std::map<std::string, std::string> attributes;  // dt, gravity, ... as written

    BaseObject* find_object(const std::string& n) const;
    Node* find_child(const std::string& n) const;
    template <typename T>
    T* find_type() const
    {
        for (auto& o : objects)
            if (auto* t = dynamic_cast<T*>(o.get())) return t;
        return nullptr;
    }
};

// The object factory: class name -> creator, as ObjectFactory::registerObject /
// createObject. A plugin's registerObjects(factory) adds its classes.
class ObjectFactory {
public:
    using Creator = std::function<std::unique_ptr<BaseObject>()>;
    struct Entry {
        std::string class_name, description, module;
        Creator create;
    };
    void register_object(const std::string& cls, const std::string& description, const std::string& module,
                         Creator c);
    bool has(const std::string& cls) const { return entries_.count(cls) != 0; }
    std::unique_ptr<BaseObject> create(const std::string& cls) const;
    std::vector<std::string> class_names() const;
    const Entry* entry(const std::string& cls) const;

private:
    std::map<std::string, Entry> entries_;
};

// Registers every component class of this library on `f`.
void register_components(ObjectFactory& f);
// The process-wide factory with this library's components registered.
ObjectFactory& default_factory();

// One simulated body: a node holding an ODE solver, its state, force field,
// mass and constraints, ready to become an sgb_scene.
struct Body {
    Node* node = nullptr;
    std::vector<double> rest;   // n x 3
    std::vector<int32_t> tets;  // E x 4
    std::vector<double> young, poisson;
    double plastic_max = 0.0, plastic_yield = 1e-4, plastic_creep = 0.9;  // TetrahedronFEMForceField plasticity
    bool update_stiffness = false;  // TetrahedronFEMForceField updateStiffnessMatrix (polar, svd)
    int von_mises_mode = 0;  // computeVonMisesStress: 0 off, 1 corotational, 2 Green strain
    int method = SGB_METHOD_LARGE;
    int precision = SGB_PRECISION_FP64;
    sgb_scene_params params{};
    std::vector<double> node_masses;  // empty: uniform vertex mass
    std::vector<int32_t> fixed;
    std::vector<double> external_force;  // n x 3 or empty
    sgb_scene_t* scene = nullptr;
    sgb_tfem_t* fem = nullptr;  // the scene's force field (owned by the scene)
};

// A parsed scene: the node tree, its host initialisation and the bodies.
class Scene {
public:
    ~Scene();
    std::unique_ptr<Node> root;
    std::vector<std::string> warnings;
    std::vector<std::string> ignored;  // "Class name (node)" of components with no effect on the step
    std::vector<Body> bodies;
    int precision_override = -1;
    double dt = 0.01;
    double gravity[3] = {0.0, -9.81, 0.0};
    double time = 0.0;
    bool device_ready = false;

    // Resolves "@path" (relative to `from`'s node) to a component; "" when
    // the path has no component part. Unqualified names are searched in the
    // node and then its ancestors.
    BaseObject* resolve_object(Node* from, const std::string& path);
    // Resolves "@path.field" to (component, field name).
    BaseObject* resolve_data(Node* from, const std::string& link, std::string* field);
    // Initialises a component (and, through links, what it reads) once.
    void ensure_init(BaseObject* o);

    // host initialisation of every component, then body assembly
    int init_host(std::string* err);
    int init_device(std::string* err);
    int animate(int n_steps, std::string* err);
    // sofa::simulation::node::reset: states back to their reset values, plastic
    // strains cleared, writers rewound, time 0 (device objects kept)
    int reset(std::string* err);
    // sofa::simulation::node::unload's counterpart for the device: every
    // body's GPU objects released; the parsed scene stays and the next
    // animate starts again from the initial state
    int unload();
    std::string describe() const;
};

// Parses the XML text of a .scn file into a Scene (no initialisation).
// Returns 0 or a negative SGB_ERR_* with the message in `err`.
int parse_scene_xml(const std::string& text, const ObjectFactory& f, Scene& out, std::string* err);

}  // namespace scn
}  // namespace sgb
