// Component layer: Data fields, links, the object factory and the node tree
// (see scene_graph.h). Component classes are in scene_components.cpp.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <sstream>

#include "scene_graph.h"

namespace sgb {
namespace scn {

// ---------------------------------------------------------------------------
// text -> values
// ---------------------------------------------------------------------------
static std::vector<double> parse_reals(const std::string& s, bool* ok)
{
    std::vector<double> v;
    const char* p = s.c_str();
    *ok = true;
    for (;;) {
        while (*p && (std::isspace((unsigned char)*p) || *p == ',' || *p == '[' || *p == ']')) ++p;
        if (!*p) break;
        char* e = nullptr;
        const double d = std::strtod(p, &e);
        if (e == p) {
            *ok = false;
            break;
        }
        v.push_back(d);
        p = e;
    }
    return v;
}

static bool parse_bool(const std::string& s)
{
    std::string l;
    for (char c : s)
        if (!std::isspace((unsigned char)c)) l += (char)std::tolower((unsigned char)c);
    return !(l.empty() || l == "0" || l == "false" || l == "no" || l == "off");
}

// ---------------------------------------------------------------------------
// BaseObject
// ---------------------------------------------------------------------------
void BaseObject::declare(const std::string& n, const std::string& def, const std::string& help)
{
    for (auto& f : fields_)
        if (f.name == n) {
            f.value = def;
            f.help = help;
            return;
        }
    fields_.push_back({n, def, help, false});
}

bool BaseObject::has_data(const std::string& n) const { return data(n) != nullptr; }

DataField* BaseObject::data(const std::string& n)
{
    for (auto& f : fields_)
        if (f.name == n) return &f;
    return nullptr;
}

const DataField* BaseObject::data(const std::string& n) const
{
    for (auto& f : fields_)
        if (f.name == n) return &f;
    return nullptr;
}

bool BaseObject::set(const std::string& n, const std::string& v)
{
    DataField* f = data(n);
    if (!f && permissive()) {
        fields_.push_back({n, v, "", true});
        return true;
    }
    if (!f) return false;
    f->value = v;
    f->is_set = true;
    return true;
}

bool BaseObject::is_set(const std::string& n) const
{
    const DataField* f = data(n);
    return f && f->is_set;
}

std::string BaseObject::get_string(const std::string& n) const
{
    const DataField* f = data(n);
    return f ? f->value : std::string();
}

std::vector<double> BaseObject::get_reals(Scene& s, const std::string& n)
{
    const DataField* f = data(n);
    if (!f) return {};
    std::string v = f->value;
    size_t b = v.find_first_not_of(" \t\r\n");
    if (b != std::string::npos && v[b] == '@') {
        std::string field;
        BaseObject* src = s.resolve_data(context, v.substr(b), &field);
        if (!src) {
            s.warnings.push_back(class_name() + " '" + name + "': cannot resolve link " + n + "=\"" + v + "\"");
            return {};
        }
        s.ensure_init(src);
        auto it = src->out_reals.find(field);
        if (it != src->out_reals.end()) return it->second;
        auto ii = src->out_ints.find(field);
        if (ii != src->out_ints.end()) return std::vector<double>(ii->second.begin(), ii->second.end());
        if (src->has_data(field)) return src->get_reals(s, field);
        s.warnings.push_back(class_name() + " '" + name + "': " + src->name + " has no Data '" + field + "'");
        return {};
    }
    bool ok = true;
    std::vector<double> r = parse_reals(v, &ok);
    if (!ok) s.warnings.push_back(class_name() + " '" + name + "': Data " + n + " is not a list of numbers");
    return r;
}

std::vector<int> BaseObject::get_ints(Scene& s, const std::string& n)
{
    std::vector<double> r = get_reals(s, n);
    std::vector<int> o;
    o.reserve(r.size());
    for (double d : r) o.push_back((int)std::llround(d));
    return o;
}

double BaseObject::get_real(Scene& s, const std::string& n)
{
    std::vector<double> r = get_reals(s, n);
    return r.empty() ? 0.0 : r[0];
}

int BaseObject::get_int(Scene& s, const std::string& n)
{
    std::vector<int> r = get_ints(s, n);
    return r.empty() ? 0 : r[0];
}

bool BaseObject::get_bool(Scene& s, const std::string& n)
{
    (void)s;
    return parse_bool(get_string(n));
}

// ---------------------------------------------------------------------------
// Node
// ---------------------------------------------------------------------------
BaseObject* Node::find_object(const std::string& n) const
{
    for (auto& o : objects)
        if (o->name == n) return o.get();
    return nullptr;
}

Node* Node::find_child(const std::string& n) const
{
    for (auto& c : children)
        if (c->name == n) return c.get();
    return nullptr;
}

// ---------------------------------------------------------------------------
// ObjectFactory
// ---------------------------------------------------------------------------
void ObjectFactory::register_object(const std::string& cls, const std::string& description, const std::string& module,
                                    Creator c)
{
    entries_[cls] = Entry{cls, description, module, std::move(c)};
}

std::unique_ptr<BaseObject> ObjectFactory::create(const std::string& cls) const
{
    auto it = entries_.find(cls);
    if (it == entries_.end()) return nullptr;
    return it->second.create();
}

std::vector<std::string> ObjectFactory::class_names() const
{
    std::vector<std::string> v;
    for (auto& e : entries_) v.push_back(e.first);
    return v;
}

const ObjectFactory::Entry* ObjectFactory::entry(const std::string& cls) const
{
    auto it = entries_.find(cls);
    return it == entries_.end() ? nullptr : &it->second;
}

ObjectFactory& default_factory()
{
    static ObjectFactory f;
    static bool done = false;
    if (!done) {
        register_components(f);
        done = true;
    }
    return f;
}

// ---------------------------------------------------------------------------
// links
// ---------------------------------------------------------------------------
static std::vector<std::string> split_path(const std::string& p)
{
    std::vector<std::string> parts;
    std::string cur;
    for (char c : p) {
        if (c == '/') {
            parts.push_back(cur);
            cur.clear();
        } else {
            cur += c;
        }
    }
    parts.push_back(cur);
    return parts;
}

BaseObject* Scene::resolve_object(Node* from, const std::string& path_in)
{
    std::string path = path_in;
    size_t b = path.find_first_not_of(" \t\r\n");
    if (b == std::string::npos) return nullptr;
    path = path.substr(b);
    while (!path.empty() && std::isspace((unsigned char)path.back())) path.pop_back();
    if (!path.empty() && path[0] == '@') path = path.substr(1);
    if (path.empty() || !from) return nullptr;
    std::vector<std::string> parts = split_path(path);
    Node* n = from;
    size_t k = 0;
    if (parts[0].empty()) {  // absolute: "/a/b"
        while (n->parent) n = n->parent;
        k = 1;
    }
    for (; k + 1 < parts.size(); ++k) {
        const std::string& p = parts[k];
        if (p == "." || p.empty()) continue;
        if (p == "..") {
            if (!n->parent) return nullptr;
            n = n->parent;
            continue;
        }
        Node* c = n->find_child(p);
        if (!c) return nullptr;
        n = c;
    }
    const std::string& last = parts.back();
    if (BaseObject* o = n->find_object(last)) return o;
    if (parts.size() == 1)  // unqualified: search the ancestors
        for (Node* a = n->parent; a; a = a->parent)
            if (BaseObject* o = a->find_object(last)) return o;
    return nullptr;
}

BaseObject* Scene::resolve_data(Node* from, const std::string& link, std::string* field)
{
    // "@path/to/object.field": the field follows the last '.' after the last '/'
    std::string l = link;
    size_t b = l.find_first_not_of(" \t\r\n@");
    if (b == std::string::npos) return nullptr;
    l = l.substr(b);
    while (!l.empty() && std::isspace((unsigned char)l.back())) l.pop_back();
    const size_t slash = l.rfind('/');
    const size_t dot = l.find('.', slash == std::string::npos ? 0 : slash + 1);
    if (dot == std::string::npos) return nullptr;
    *field = l.substr(dot + 1);
    return resolve_object(from, l.substr(0, dot));
}

void Scene::ensure_init(BaseObject* o)
{
    if (!o || o->initialized || o->initializing) return;
    o->initializing = true;
    o->init(*this);
    o->initializing = false;
    o->initialized = true;
}

Scene::~Scene()
{
    for (auto& b : bodies)
        if (b.scene) sgb_scene_destroy(b.scene);
}

// ---------------------------------------------------------------------------
// description (JSON)
// ---------------------------------------------------------------------------
static std::string jstr(const std::string& s)
{
    std::string o = "\"";
    for (char c : s) {
        if (c == '"' || c == '\\') {
            o += '\\';
            o += c;
        } else if (c == '\n') {
            o += "\\n";
        } else if ((unsigned char)c < 0x20) {
            o += ' ';
        } else {
            o += c;
        }
    }
    return o + "\"";
}

static void describe_node(const Node* n, std::ostringstream& os)
{
    os << "{\"name\":" << jstr(n->name) << ",\"objects\":[";
    for (size_t i = 0; i < n->objects.size(); ++i) {
        const BaseObject* o = n->objects[i].get();
        os << (i ? "," : "") << "{\"class\":" << jstr(o->class_name()) << ",\"name\":" << jstr(o->name);
        if (!o->template_name.empty()) os << ",\"template\":" << jstr(o->template_name);
        if (o->ignored()) os << ",\"ignored\":true";
        os << ",\"data\":{";
        bool first = true;
        for (auto& f : o->fields())
            if (f.is_set) {
                os << (first ? "" : ",") << jstr(f.name) << ":" << jstr(f.value);
                first = false;
            }
        os << "}}";
    }
    os << "],\"children\":[";
    for (size_t i = 0; i < n->children.size(); ++i) {
        if (i) os << ",";
        describe_node(n->children[i].get(), os);
    }
    os << "]}";
}

std::string Scene::describe() const
{
    std::ostringstream os;
    os.precision(17);
    os << "{\"dt\":" << dt << ",\"gravity\":[" << gravity[0] << "," << gravity[1] << "," << gravity[2] << "]";
    os << ",\"bodies\":[";
    for (size_t i = 0; i < bodies.size(); ++i) {
        const Body& b = bodies[i];
        os << (i ? "," : "") << "{\"node\":" << jstr(b.node ? b.node->name : "") << ",\"n_nodes\":" << b.rest.size() / 3
           << ",\"n_tets\":" << b.tets.size() / 4 << ",\"method\":" << b.method << ",\"precision\":" << b.precision
           << ",\"n_fixed\":" << b.fixed.size() << ",\"fix_all\":" << b.params.fix_all
           << ",\"uniform_vertex_mass\":" << (b.node_masses.empty() ? b.params.vertex_mass : 0.0)
           << ",\"dt\":" << b.params.dt << ",\"rayleigh_stiffness\":" << b.params.rayleigh_stiffness
           << ",\"rayleigh_mass\":" << b.params.rayleigh_mass << ",\"vdamping\":" << b.params.vdamping
           << ",\"cg_iterations\":" << b.params.cg_iterations << ",\"cg_tolerance\":" << b.params.cg_tolerance
           << ",\"cg_threshold\":" << b.params.cg_threshold << ",\"mass_first\":" << b.params.mass_first << "}";
    }
    os << "],\"ignored\":[";
    for (size_t i = 0; i < ignored.size(); ++i) os << (i ? "," : "") << jstr(ignored[i]);
    os << "],\"warnings\":[";
    for (size_t i = 0; i < warnings.size(); ++i) os << (i ? "," : "") << jstr(warnings[i]);
    os << "],\"root\":";
    if (root) describe_node(root.get(), os);
    else os << "null";
    os << "}";
    return os.str();
}

}  // namespace scn
}  // namespace sgb
