// Minimal XML reader for SOFA scene files (.scn): elements, attributes,
// comments, the XML declaration and the five predefined entities. <Node>
// elements become nodes, every other element a component created through
// the object factory (the role SceneLoaderXML plays in the reference,
// Sofa/framework/Simulation/Common/src/sofa/simulation/common/SceneLoaderXML.cpp,
// which needs TinyXML2).
#include <cctype>
#include <cstring>
#include <set>
#include <string>

#include "scene_graph.h"

namespace sgb {
namespace scn {

namespace {

// Components of the reference's soft-body scenes that have no effect on the
// implicit FEM step: plugin declarations, visual and collision-pipeline
// components, surface extraction for rendering. They are accepted and listed.
const std::set<std::string>& ignored_classes()
{
    static const std::set<std::string> s = {
        "RequiredPlugin", "VisualStyle", "DefaultVisualManagerLoop", "CollisionPipeline", "BruteForceBroadPhase",
        "BVHNarrowPhase", "CollisionResponse", "DiscreteIntersection", "MinProximityIntersection",
        "LocalMinDistance", "NewProximityIntersection", "OglModel", "VisualModel", "IdentityMapping",
        "TriangleSetTopologyContainer", "TriangleSetTopologyModifier", "TriangleSetGeometryAlgorithms",
        "Tetra2TriangleTopologicalMapping", "BlockGaussSeidelConstraintSolver", "GenericConstraintSolver",
        "InfoComponent", "OglGrid", "OglLabel", "LightManager", "DirectionalLight", "PositionalLight",
        "InteractiveCamera", "BackgroundSetting", "ViewerSetting", "AttachBodyButtonSetting",
        "TriangleCollisionModel", "LineCollisionModel", "PointCollisionModel", "SphereCollisionModel",
        "DefaultPipeline", "DefaultContactManager", "BruteForceDetection"};
    return s;
}

class IgnoredObject : public BaseObject {
public:
    explicit IgnoredObject(const std::string& cls) : BaseObject(cls) {}
    bool ignored() const override { return true; }
};

struct Attr {
    std::string name, value;
};

struct Parser {
    const std::string& t;
    size_t i = 0;
    std::string err;

    explicit Parser(const std::string& text) : t(text) {}

    bool eof() const { return i >= t.size(); }
    void skip_ws()
    {
        while (!eof() && std::isspace((unsigned char)t[i])) ++i;
    }
    bool starts(const char* s) const { return t.compare(i, std::strlen(s), s) == 0; }

    int line() const
    {
        int l = 1;
        for (size_t k = 0; k < i && k < t.size(); ++k)
            if (t[k] == '\n') ++l;
        return l;
    }
    bool fail(const std::string& m)
    {
        if (err.empty()) err = "scene XML, line " + std::to_string(line()) + ": " + m;
        return false;
    }

    // skips text, comments, declarations and processing instructions up to
    // the next element tag ('<' of a start or end tag)
    bool skip_misc()
    {
        for (;;) {
            while (!eof() && t[i] != '<') ++i;
            if (eof()) return true;
            if (starts("<!--")) {
                size_t e = t.find("-->", i + 4);
                if (e == std::string::npos) return fail("unterminated comment");
                i = e + 3;
            } else if (starts("<?")) {
                size_t e = t.find("?>", i + 2);
                if (e == std::string::npos) return fail("unterminated declaration");
                i = e + 2;
            } else if (starts("<!")) {
                size_t e = t.find('>', i + 2);
                if (e == std::string::npos) return fail("unterminated markup declaration");
                i = e + 1;
            } else {
                return true;
            }
        }
    }

    static std::string decode(const std::string& v)
    {
        std::string o;
        for (size_t k = 0; k < v.size(); ++k) {
            if (v[k] == '&') {
                static const struct {
                    const char* e;
                    char c;
                } ents[] = {{"&lt;", '<'}, {"&gt;", '>'}, {"&amp;", '&'}, {"&quot;", '"'}, {"&apos;", '\''}};
                bool done = false;
                for (auto& en : ents)
                    if (v.compare(k, std::strlen(en.e), en.e) == 0) {
                        o += en.c;
                        k += std::strlen(en.e) - 1;
                        done = true;
                        break;
                    }
                if (!done) o += v[k];
            } else {
                o += v[k];
            }
        }
        return o;
    }

    bool name(std::string& n)
    {
        size_t s = i;
        while (!eof() && (std::isalnum((unsigned char)t[i]) || t[i] == '_' || t[i] == '-' || t[i] == '.' ||
                          t[i] == ':'))
            ++i;
        if (i == s) return fail("expected a name");
        n = t.substr(s, i - s);
        return true;
    }

    // parses "<Name a="v" ...>" or "<Name .../>"; `empty` = self-closing
    bool start_tag(std::string& tag, std::vector<Attr>& attrs, bool& empty)
    {
        ++i;  // '<'
        if (!name(tag)) return false;
        for (;;) {
            skip_ws();
            if (eof()) return fail("unterminated tag <" + tag + ">");
            if (starts("/>")) {
                i += 2;
                empty = true;
                return true;
            }
            if (t[i] == '>') {
                ++i;
                empty = false;
                return true;
            }
            Attr a;
            if (!name(a.name)) return false;
            skip_ws();
            if (eof() || t[i] != '=') return fail("expected '=' after attribute " + a.name);
            ++i;
            skip_ws();
            if (eof() || (t[i] != '"' && t[i] != '\'')) return fail("expected a quoted value for " + a.name);
            const char q = t[i++];
            size_t e = t.find(q, i);
            if (e == std::string::npos) return fail("unterminated value of " + a.name);
            a.value = decode(t.substr(i, e - i));
            i = e + 1;
            attrs.push_back(std::move(a));
        }
    }
};

int build_element(Parser& p, const ObjectFactory& f, Scene& sc, Node* parent, std::unique_ptr<Node>* root_out,
                  std::string* err, int depth)
{
    if (depth > 256) {
        *err = "scene XML: nesting deeper than 256 levels";
        return SGB_ERR_INVALID_ARGUMENT;
    }
    std::string tag;
    std::vector<Attr> attrs;
    bool empty = false;
    if (!p.start_tag(tag, attrs, empty)) {
        *err = p.err;
        return SGB_ERR_INVALID_ARGUMENT;
    }
    Node* node = nullptr;
    if (tag == "Node") {
        auto n = std::make_unique<Node>();
        n->parent = parent;
        for (auto& a : attrs) {
            if (a.name == "name")
                n->name = a.value;
            else
                n->attributes[a.name] = a.value;
        }
        node = n.get();
        if (parent)
            parent->children.push_back(std::move(n));
        else
            *root_out = std::move(n);
    } else {
        if (!parent) {
            *err = "scene XML: the root element must be <Node>, found <" + tag + ">";
            return SGB_ERR_INVALID_ARGUMENT;
        }
        std::unique_ptr<BaseObject> o;
        if (f.has(tag)) {
            o = f.create(tag);
        } else if (ignored_classes().count(tag)) {
            o = std::make_unique<IgnoredObject>(tag);
        } else {
            *err = "scene XML, line " + std::to_string(p.line()) + ": unknown component <" + tag +
                   "> (not part of the implicit tetrahedral-FEM component set)";
            return SGB_ERR_NOT_SUPPORTED;
        }
        o->context = parent;
        for (auto& a : attrs) {
            if (a.name == "name") {
                o->name = a.value;
            } else if (a.name == "template") {
                o->template_name = a.value;
            } else if (!o->set(a.name, a.value) && !o->ignored()) {
                sc.warnings.push_back(tag + (o->name.empty() ? "" : " '" + o->name + "'") + ": attribute '" +
                                      a.name + "' is not used");
            }
        }
        if (o->name.empty()) o->name = tag;
        if (o->ignored())
            sc.ignored.push_back(tag + " '" + o->name + "' (node " + (parent->name.empty() ? "?" : parent->name) +
                                 ")");
        parent->objects.push_back(std::move(o));
    }
    if (empty) return SGB_OK;
    // children up to the matching end tag
    for (;;) {
        if (!p.skip_misc()) {
            *err = p.err;
            return SGB_ERR_INVALID_ARGUMENT;
        }
        if (p.eof()) {
            *err = "scene XML: missing </" + tag + ">";
            return SGB_ERR_INVALID_ARGUMENT;
        }
        if (p.starts("</")) {
            p.i += 2;
            std::string end;
            if (!p.name(end)) {
                *err = p.err;
                return SGB_ERR_INVALID_ARGUMENT;
            }
            p.skip_ws();
            if (p.eof() || p.t[p.i] != '>' || end != tag) {
                *err = "scene XML, line " + std::to_string(p.line()) + ": </" + end + "> does not close <" + tag + ">";
                return SGB_ERR_INVALID_ARGUMENT;
            }
            ++p.i;
            return SGB_OK;
        }
        if (!node) {
            *err = "scene XML, line " + std::to_string(p.line()) + ": component <" + tag + "> has child elements";
            return SGB_ERR_INVALID_ARGUMENT;
        }
        int rc = build_element(p, f, sc, node, root_out, err, depth + 1);
        if (rc) return rc;
    }
}

}  // namespace

int parse_scene_xml(const std::string& text, const ObjectFactory& f, Scene& out, std::string* err)
{
    Parser p(text);
    if (!p.skip_misc()) {
        *err = p.err;
        return SGB_ERR_INVALID_ARGUMENT;
    }
    if (p.eof()) {
        *err = "scene XML: no root element";
        return SGB_ERR_INVALID_ARGUMENT;
    }
    int rc = build_element(p, f, out, nullptr, &out.root, err, 0);
    if (rc) return rc;
    if (!p.skip_misc()) {
        *err = p.err;
        return SGB_ERR_INVALID_ARGUMENT;
    }
    if (!p.eof()) {
        *err = "scene XML: content after the root element";
        return SGB_ERR_INVALID_ARGUMENT;
    }
    if (!out.root) {
        *err = "scene XML: no root <Node>";
        return SGB_ERR_INVALID_ARGUMENT;
    }
    return SGB_OK;
}

}  // namespace scn
}  // namespace sgb
