// Component classes of the implicit tetrahedral-FEM step, with the
// reference's class names and Data names/defaults, and the scene assembly
// that turns a node holding an EulerImplicitSolver into a library scene.
#include <algorithm>
#include <cmath>
#include <fstream>
#include <set>
#include <sstream>

#include "scene_graph.h"

namespace sgb {
namespace scn {

namespace {

// Components that accept any attribute silently (drawing options, topology
// bookkeeping) besides their declared Data.
class PermissiveObject : public BaseObject {
public:
    using BaseObject::BaseObject;
    bool permissive() const override { return true; }
};

// ---- RegularGridTopology ----------------------------------------------------
// Node numbering index = nx*(ny*k + j) + i and hexahedron corner order of
// GridTopology (Sofa/Component/Topology/Container/Grid/src/sofa/component/
// topology/container/grid/GridTopology.cpp:352-356, :391-398); positions
// min + (max-min)/(n-1) * (i,j,k) (RegularGridTopology.cpp:165-168).
class RegularGridTopology : public BaseObject {
public:
    RegularGridTopology() : BaseObject("RegularGridTopology")
    {
        declare("n", "2 2 2", "grid resolution (nodes per axis)");
        declare("min", "0 0 0", "lower corner");
        declare("max", "1 1 1", "upper corner");
        declare("p0", "0 0 0", "offset (unused when min/max are given)");
        declare("computeHexaList", "1", "");
        declare("computeQuadList", "1", "");
        declare("computeTriangleList", "1", "");
        declare("computeEdgeList", "1", "");
        declare("drawEdges", "0", "");
    }
    void init(Scene& s) override
    {
        std::vector<int> n = get_ints(s, "n");
        std::vector<double> lo = get_reals(s, "min"), hi = get_reals(s, "max");
        if (n.size() != 3 || lo.size() != 3 || hi.size() != 3) {
            s.warnings.push_back("RegularGridTopology '" + name + "': n, min and max need 3 values each");
            return;
        }
        const int nx = std::max(n[0], 1), ny = std::max(n[1], 1), nz = std::max(n[2], 1);
        double d[3];
        const int nn[3] = {nx, ny, nz};
        for (int a = 0; a < 3; ++a) d[a] = nn[a] > 1 ? (hi[a] - lo[a]) / (nn[a] - 1) : 0.0;
        std::vector<double>& pos = out_reals["position"];
        pos.resize((size_t)nx * ny * nz * 3);
        for (int k = 0; k < nz; ++k)
            for (int j = 0; j < ny; ++j)
                for (int i = 0; i < nx; ++i) {
                    const size_t id = (size_t)nx * ((size_t)ny * k + j) + i;
                    pos[3 * id] = lo[0] + d[0] * i;
                    pos[3 * id + 1] = lo[1] + d[1] * j;
                    pos[3 * id + 2] = lo[2] + d[2] * k;
                }
        std::vector<int>& hx = out_ints["hexahedra"];
        hx.clear();
        if (nx > 1 && ny > 1 && nz > 1) {
            auto p = [&](int a, int b, int c) { return nx * (ny * c + b) + a; };
            for (int z = 0; z < nz - 1; ++z)
                for (int y = 0; y < ny - 1; ++y)
                    for (int x = 0; x < nx - 1; ++x) {
                        const int c[8] = {p(x, y, z),         p(x + 1, y, z),         p(x + 1, y + 1, z),
                                          p(x, y + 1, z),     p(x, y, z + 1),         p(x + 1, y, z + 1),
                                          p(x + 1, y + 1, z + 1), p(x, y + 1, z + 1)};
                        hx.insert(hx.end(), c, c + 8);
                    }
        }
        out_ints["n"] = {nx, ny, nz};
    }
};

// ---- Hexa2TetraTopologicalMapping --------------------------------------------
// Six tetrahedra per hexahedron with the optional corner swapping by grid
// parity (Sofa/Component/Topology/Mapping/src/sofa/component/topology/
// mapping/Hexa2TetraTopologicalMapping.cpp:104-199): swapped cells mirror
// their corners along x (even cell x), y (odd cell y) and z (odd cell z),
// and cells with an odd number of mirrors use the second corner pattern.
class Hexa2TetraTopologicalMapping : public BaseObject {
public:
    Hexa2TetraTopologicalMapping() : BaseObject("Hexa2TetraTopologicalMapping")
    {
        declare("input", "", "input hexahedral topology");
        declare("output", "", "output tetrahedral topology");
        declare("swapping", "0", "swap corners by grid parity");
    }
    void init(Scene& s) override
    {
        BaseObject* in = s.resolve_object(context, get_string("input"));
        BaseObject* out = s.resolve_object(context, get_string("output"));
        if (!in || !out) {
            s.warnings.push_back("Hexa2TetraTopologicalMapping: cannot resolve input/output");
            return;
        }
        s.ensure_init(in);
        auto hit = in->out_ints.find("hexahedra");
        if (hit == in->out_ints.end()) {
            s.warnings.push_back("Hexa2TetraTopologicalMapping: input '" + in->name + "' has no hexahedra");
            return;
        }
        const std::vector<int>& hx = hit->second;
        int cx = 2, cy = 1;
        auto nit = in->out_ints.find("n");
        if (nit != in->out_ints.end()) {
            cx = std::max(nit->second[0] - 1, 1);
            cy = std::max(nit->second[1] - 1, 1);
        }
        static const int plain[6][4] = {{0, 5, 1, 6}, {0, 1, 3, 6}, {1, 3, 6, 2},
                                        {6, 3, 0, 7}, {6, 7, 0, 5}, {7, 5, 4, 0}};
        static const int swapped_t[6][4] = {{0, 5, 6, 1}, {0, 1, 6, 3}, {1, 3, 2, 6},
                                            {6, 3, 7, 0}, {6, 7, 5, 0}, {7, 5, 0, 4}};
        static const int xe[4][2] = {{0, 1}, {4, 5}, {3, 2}, {7, 6}};
        static const int ye[4][2] = {{4, 7}, {5, 6}, {1, 2}, {0, 3}};
        static const int ze[4][2] = {{4, 0}, {5, 1}, {6, 2}, {7, 3}};
        const bool swapping = get_bool(s, "swapping");
        std::vector<int> tets;
        const size_t H = hx.size() / 8;
        tets.reserve(H * 24);
        for (size_t h = 0; h < H; ++h) {
            int c[8];
            for (int k = 0; k < 8; ++k) c[k] = hx[8 * h + k];
            bool sw = false;
            if (swapping) {
                if (!((h % cx) & 1)) {
                    for (auto& e : xe) std::swap(c[e[0]], c[e[1]]);
                    sw = !sw;
                }
                if (((h / cx) % cy) & 1) {
                    for (auto& e : ye) std::swap(c[e[0]], c[e[1]]);
                    sw = !sw;
                }
                if ((h / ((size_t)cx * cy)) & 1) {
                    for (auto& e : ze) std::swap(c[e[0]], c[e[1]]);
                    sw = !sw;
                }
            }
            const int(*pat)[4] = sw ? swapped_t : plain;
            for (int t = 0; t < 6; ++t)
                for (int k = 0; k < 4; ++k) tets.push_back(c[pat[t][k]]);
        }
        out->out_ints["tetrahedra"] = tets;
        auto pit = in->out_reals.find("position");
        if (pit != in->out_reals.end()) out->out_reals["position"] = pit->second;
    }
};

// ---- TetrahedronSetTopologyContainer ------------------------------------------
class TetrahedronSetTopologyContainer : public PermissiveObject {
public:
    TetrahedronSetTopologyContainer() : PermissiveObject("TetrahedronSetTopologyContainer")
    {
        declare("tetrahedra", "", "tetrahedra (4 node indices each)");
        declare("position", "", "initial positions");
        declare("src", "", "container (or loader) to copy the topology from");
    }
    void init(Scene& s) override
    {
        if (is_set("tetrahedra")) out_ints["tetrahedra"] = get_ints(s, "tetrahedra");
        if (is_set("position")) out_reals["position"] = get_reals(s, "position");
        if (is_set("src")) {
            if (BaseObject* src = s.resolve_object(context, get_string("src"))) {
                s.ensure_init(src);
                auto t = src->out_ints.find("tetrahedra");
                if (t != src->out_ints.end()) out_ints["tetrahedra"] = t->second;
                auto p = src->out_reals.find("position");
                if (p != src->out_reals.end()) out_reals["position"] = p->second;
            } else {
                s.warnings.push_back("TetrahedronSetTopologyContainer '" + name + "': cannot resolve src");
            }
        }
        // a topological mapping of this node that outputs here fills it
        for (auto& o : context->objects)
            if (o->class_name() == "Hexa2TetraTopologicalMapping" &&
                s.resolve_object(context, o->get_string("output")) == this)
                s.ensure_init(o.get());
    }
};

// ---- MechanicalObject ---------------------------------------------------------
class MechanicalObject : public BaseObject {
public:
    MechanicalObject() : BaseObject("MechanicalObject")
    {
        declare("position", "", "positions");
        declare("velocity", "", "velocities");
        declare("rest_position", "", "rest positions");
        declare("force", "", "forces");
        declare("externalForce", "", "external forces (accumulateForce, MechanicalObject.inl:1357-1376)");
        declare("derivX", "", "");
        declare("free_position", "", "");
        declare("free_velocity", "", "");
        declare("showObject", "0", "");
        declare("showObjectScale", "0.1", "");
        declare("showIndices", "0", "");
        declare("showIndicesScale", "0.02", "");
        declare("showColor", "", "");
        declare("drawMode", "0", "");
    }
    void init(Scene& s) override
    {
        std::vector<double> x = get_reals(s, "position");
        if (x.empty()) {
            // from the node's topology: a container or a grid
            for (auto& o : context->objects) {
                if (o.get() == this) continue;
                if (o->class_name() == "TetrahedronSetTopologyContainer" ||
                    o->class_name() == "RegularGridTopology") {
                    s.ensure_init(o.get());
                    auto p = o->out_reals.find("position");
                    if (p != o->out_reals.end() && !p->second.empty()) {
                        x = p->second;
                        break;
                    }
                }
            }
        }
        if (x.size() % 3) {
            s.warnings.push_back("MechanicalObject '" + name + "': position is not a list of 3-vectors");
            x.resize(x.size() - x.size() % 3);
        }
        out_reals["position"] = x;
        std::vector<double> r = get_reals(s, "rest_position");
        out_reals["rest_position"] = r.size() == x.size() ? r : x;
        std::vector<double> v = get_reals(s, "velocity");
        out_reals["velocity"] = v.size() == x.size() ? v : std::vector<double>(x.size(), 0.0);
        std::vector<double> fe = get_reals(s, "externalForce");
        if (fe.size() == x.size()) out_reals["externalForce"] = fe;
    }
};

// ---- BoxROI -------------------------------------------------------------------
// Indices of the points inside any of the boxes (xmin ymin zmin xmax ymax
// zmax), bounds inclusive, in ascending order; the points default to the
// node's MechanicalObject rest positions
// (Sofa/Component/Engine/Select/src/sofa/component/engine/select/BoxROI.inl).
class BoxROI : public PermissiveObject {
public:
    BoxROI() : PermissiveObject("BoxROI")
    {
        declare("box", "", "boxes: xmin ymin zmin xmax ymax zmax each");
        declare("position", "", "points to test (default: the node's rest positions)");
        declare("indices", "", "output: indices of the points inside");
    }
    void init(Scene& s) override
    {
        std::vector<double> p = get_reals(s, "position");
        if (!is_set("position") || p.empty()) {
            p.clear();
            for (auto& o : context->objects)
                if (o->class_name() == "MechanicalObject") {
                    s.ensure_init(o.get());
                    p = o->out_reals["rest_position"];
                    break;
                }
        }
        std::vector<double> b = get_reals(s, "box");
        std::vector<int> idx;
        for (size_t k = 0; k + 5 < b.size(); k += 6) {
            double lo[3] = {b[k], b[k + 1], b[k + 2]}, hi[3] = {b[k + 3], b[k + 4], b[k + 5]};
            for (int a = 0; a < 3; ++a)
                if (lo[a] > hi[a]) std::swap(lo[a], hi[a]);
            for (size_t i = 0; i < p.size() / 3; ++i) {
                bool in = true;
                for (int a = 0; a < 3; ++a) in = in && p[3 * i + a] >= lo[a] && p[3 * i + a] <= hi[a];
                if (in) idx.push_back((int)i);
            }
        }
        std::sort(idx.begin(), idx.end());
        idx.erase(std::unique(idx.begin(), idx.end()), idx.end());
        out_ints["indices"] = idx;
    }
};

// ---- FixedProjectiveConstraint --------------------------------------------------
// Data of FixedProjectiveConstraint.inl:39-48 (indices default {0}).
class FixedProjectiveConstraint : public PermissiveObject {
public:
    explicit FixedProjectiveConstraint(const char* cls = "FixedProjectiveConstraint") : PermissiveObject(cls)
    {
        declare("indices", "0", "indices of the fixed points");
        declare("fixAll", "0", "fix every point");
        declare("activate_projectVelocity", "0", "also project velocities");
        declare("showObject", "1", "");
        declare("drawSize", "0", "");
        declare("mstate", "", "link to the MechanicalObject");
    }
    void init(Scene& s) override { out_ints["indices"] = get_ints(s, "indices"); }
};

// ---- masses -----------------------------------------------------------------------
class UniformMass : public PermissiveObject {
public:
    UniformMass() : PermissiveObject("UniformMass")
    {
        declare("vertexMass", "1", "mass of each particle");
        declare("totalMass", "1", "total mass (vertexMass = totalMass / n)");
        declare("indices", "", "");
        declare("preserveTotalMass", "0", "");
        declare("rayleighMass", "0", "Rayleigh mass damping of the component (BaseMass)");
        declare("separateGravity", "0", "");
        declare("filename", "unused", "");
    }
};

class DiagonalMass : public PermissiveObject {
public:
    DiagonalMass() : PermissiveObject("DiagonalMass")
    {
        declare("vertexMass", "", "per-point masses");
        declare("massDensity", "1", "mass density");
        declare("totalMass", "1", "total mass");
        declare("computeMassOnRest", "1", "");
        declare("rayleighMass", "0", "Rayleigh mass damping of the component (BaseMass)");
        declare("separateGravity", "0", "");
    }
};

// ---- TetrahedronFEMForceField --------------------------------------------------------
// Data of TetrahedronFEMForceField.inl:41-67 and BaseLinearElasticityFEMForceField.inl:33-34.
class TetrahedronFEMForceField : public PermissiveObject {
public:
    TetrahedronFEMForceField() : PermissiveObject("TetrahedronFEMForceField")
    {
        declare("youngModulus", "5000", "Young's modulus (one value or one per element)");
        declare("poissonRatio", "0.45", "Poisson ratio (one value or one per element)");
        declare("method", "large", "small, large (QR), polar or svd");
        declare("initialPoints", "", "");
        declare("localStiffnessFactor", "", "per-element stiffness factors");
        declare("updateStiffnessMatrix", "0", "");
        declare("computeGlobalMatrix", "0", "");
        declare("assembling", "0", "alias of computeGlobalMatrix");
        declare("plasticMaxThreshold", "0", "");
        declare("plasticYieldThreshold", "0.0001", "");
        declare("plasticCreep", "0.9", "");
        declare("gatherPt", "", "");
        declare("gatherBsize", "", "");
        declare("computeVonMisesStress", "0", "");
        declare("updateStiffness", "0", "");
        declare("rayleighStiffness", "0", "Rayleigh stiffness damping of the component (BaseForceField)");
        declare("topology", "", "");
    }
};

// ---- solvers ----------------------------------------------------------------------------
// Data of EulerImplicitSolver.cpp:40-51 and CGLinearSolver.inl:34-46.
class EulerImplicitSolver : public PermissiveObject {
public:
    EulerImplicitSolver() : PermissiveObject("EulerImplicitSolver")
    {
        declare("rayleighStiffness", "0", "");
        declare("rayleighMass", "0", "");
        declare("vdamping", "0", "");
        declare("firstOrder", "0", "");
        declare("trapezoidalScheme", "0", "");
        declare("solveConstraint", "0", "");
        declare("threadSafeVisitor", "0", "");
        declare("computeResidual", "0", "");
    }
};

class CGLinearSolver : public PermissiveObject {
public:
    CGLinearSolver() : PermissiveObject("CGLinearSolver")
    {
        declare("iterations", "25", "");
        declare("tolerance", "1e-5", "");
        declare("threshold", "1e-5", "");
        declare("warmStart", "0", "");
        declare("graph", "", "");
    }
};

// PCGLinearSolver (PCGLinearSolver.inl:36-48): matrix-free PCG, optionally
// preconditioned by a linked JacobiPreconditioner; PreconditionedMatrixFreeSystem
// (PreconditionedMatrixFreeSystem.inl:31-34) sets how often the
// preconditioner is assembled.
class PCGLinearSolver : public PermissiveObject {
public:
    PCGLinearSolver() : PermissiveObject("PCGLinearSolver")
    {
        declare("iterations", "25", "maximum number of iterations");
        declare("tolerance", "1e-5", "stop when r.z <= tolerance * b.b");
        declare("use_precond", "1", "use the preconditioner");
        declare("preconditioner", "", "link to the preconditioner (JacobiPreconditioner)");
        declare("update_step", "1", "deprecated: assemblingRate of PreconditionedMatrixFreeSystem");
        declare("graph", "", "");
    }
};

class JacobiPreconditioner : public PermissiveObject {
public:
    JacobiPreconditioner() : PermissiveObject("JacobiPreconditioner") {}
};

class PreconditionedMatrixFreeSystem : public PermissiveObject {
public:
    PreconditionedMatrixFreeSystem() : PermissiveObject("PreconditionedMatrixFreeSystem")
    {
        declare("assemblingRate", "1", "the preconditioner is assembled every this many steps");
    }
};

class DefaultAnimationLoop : public PermissiveObject {
public:
    DefaultAnimationLoop() : PermissiveObject("DefaultAnimationLoop") {}
};

class TopologyBookkeeping : public PermissiveObject {
public:
    explicit TopologyBookkeeping(const char* cls) : PermissiveObject(cls) {}
};

template <typename T>
ObjectFactory::Creator make()
{
    return [] { return std::unique_ptr<BaseObject>(new T()); };
}

void init_tree(Scene& s, Node* n)
{
    for (auto& o : n->objects) s.ensure_init(o.get());
    for (auto& c : n->children) init_tree(s, c.get());
}

// Precision from a template name: float vectors (Vec3f, CudaVec3f) run the
// mixed path, double (Vec3d, Vec3, CudaVec3d) the FP64 reference-rounding path.
int precision_of(const std::string& tpl, int fallback)
{
    if (tpl.empty()) return fallback;
    if (tpl.find("3f") != std::string::npos) return SGB_PRECISION_MIXED;
    if (tpl.find("3d") != std::string::npos || tpl == "Vec3" || tpl == "CudaVec3") return SGB_PRECISION_FP64;
    return fallback;
}

int unsupported(std::string* err, const std::string& m)
{
    *err = m;
    return SGB_ERR_NOT_SUPPORTED;
}

// WriteState (Sofa/Component/Playback/src/sofa/component/playback/
// WriteState.inl: Data 36-46, init 73-220, handleEvent 240-380): at the
// beginning of every step whose time reaches the next export time (or, once
// the first export is done, the previous one plus the period) it appends
// "T= t" and the selected vectors of its node's MechanicalObject, each as
// "  X= x0 y0 z0 x1 y1 z1 ..." in default stream formatting (Vec and vector
// stream operators, Vec.h:765-771, vector_T.h:121-130). Without `time` and
// `period` it writes every step from t = 0. The kinetic-energy stop
// (stopAt) and the force vector (writeF) are not available.
class WriteState : public PermissiveObject {
public:
    WriteState() : PermissiveObject("WriteState")
    {
        declare("filename", "", "output file name");
        declare("writeX", "1", "flag enabling output of X vector");
        declare("writeX0", "0", "flag enabling output of X0 vector");
        declare("writeV", "0", "flag enabling output of V vector");
        declare("writeF", "0", "flag enabling output of F vector (not available)");
        declare("time", "", "set time to write outputs (by default export at t=0)");
        declare("period", "0", "period between outputs");
        declare("DOFsX", "", "set the position DOFs to write");
        declare("DOFsV", "", "set the velocity DOFs to write");
        declare("stopAt", "0", "stop the simulation when the given threshold is reached (not available)");
        declare("keperiod", "0", "set the period to measure the kinetic energy increase");
    }

    void init(Scene& s) override
    {
        valid = true;
        periodic = false;
        next = 0;
        last_time = 0.0;
        first_export = false;
        times = is_set("time") ? get_reals(s, "time") : std::vector<double>();
        period = get_real(s, "period");
        if (is_set("period")) {
            periodic = true;
            if (times.empty()) times.assign(1, 0.0);
            if (times.size() > 1) times.resize(1);
        } else if (!is_set("time")) {
            period = s.dt;
            periodic = true;
        }
        if (!is_set("time")) {
            times.assign(1, 0.0);
        } else {
            for (size_t i = 0; i < times.size(); ++i)
                if (times[i] < 0.0 || (times[i] == 0.0 && i > 0)) {
                    s.warnings.push_back("WriteState '" + name + "': export times must be positive; no export");
                    valid = false;
                }
        }
        path = get_string("filename");
        if (path.empty()) path = "defaultExportFile";
    }

    // WriteState::reset (WriteState.inl:231-238): the next record is again
    // the first export time
    void rewind()
    {
        next = 0;
        last_time = 0.0;
    }

    // AnimateBeginEvent at simulation time t: writes the state if due.
    int begin_step(Scene& s, double t, std::string* err)
    {
        if (!valid) return SGB_OK;
        if (get_bool(s, "writeF")) return unsupported(err, "WriteState '" + name + "': writeF is not available");
        if (get_real(s, "stopAt") > 0.0)
            return unsupported(err, "WriteState '" + name + "': stopAt (kinetic-energy stop) is not available");
        bool write_now = false;
        const double eps = 0.1 * s.dt;
        if (next < times.size()) {
            last_time = times[next];
            if (t > last_time || std::fabs(t - last_time) < eps) {
                write_now = true;
                first_export = true;
                ++next;
            }
        } else if (first_export && periodic) {
            const double nt = last_time + period;
            if (t > nt || std::fabs(t - nt) < eps) {
                write_now = true;
                last_time += period;
            }
        }
        if (!write_now) return SGB_OK;
        Body* body = nullptr;
        for (auto& b : s.bodies)
            if (b.node == context) body = &b;
        if (!body) return unsupported(err, "WriteState '" + name + "': no simulated MechanicalObject in its node");
        if (!out.is_open()) {
            out.open(path, std::ios::out | std::ios::trunc);
            if (!out.is_open()) return unsupported(err, "WriteState '" + name + "': cannot create " + path);
        }
        const size_t n = body->rest.size() / 3;
        std::vector<double> x(3 * n), v(3 * n);
        int rc = sgb_scene_get_state(body->scene, x.data(), v.data());
        if (rc) {
            *err = sgb_last_error();
            return rc;
        }
        out << "T= " << t << "\n";
        if (get_bool(s, "writeX")) write_vec("  X= ", x);
        if (get_bool(s, "writeX0")) write_vec("  X0= ", body->rest);
        if (get_bool(s, "writeV")) write_vec("  V= ", v);
        out.flush();
        return SGB_OK;
    }

private:
    void write_vec(const char* tag, const std::vector<double>& a)
    {
        out << tag;
        for (size_t i = 0; i < a.size(); ++i) {
            if (i) out << " ";
            out << a[i];
        }
        out << "\n";
    }

    bool valid = false, periodic = false, first_export = false;
    std::vector<double> times;
    double period = 0.0, last_time = 0.0;
    size_t next = 0;
    std::string path;
    std::ofstream out;
};


// Lumped tetrahedral masses (DiagonalMass.inl:332-376 for massDensity,
// :1221-1257 for totalMass: masses at density 1, then scaled by
// totalMass / their sum).
std::vector<double> diagonal_masses(Scene& s, BaseObject* dm, const std::vector<double>& rest,
                                    const std::vector<int32_t>& tets)
{
    const size_t N = rest.size() / 3;
    auto lumped = [&](double density) {
        std::vector<double> m(N, 0.0);
        for (size_t e = 0; e < tets.size() / 4; ++e) {
            const int32_t* t = &tets[4 * e];
            double a[3], b[3], c[3];
            for (int k = 0; k < 3; ++k) {
                a[k] = rest[3 * (size_t)t[1] + k] - rest[3 * (size_t)t[0] + k];
                b[k] = rest[3 * (size_t)t[2] + k] - rest[3 * (size_t)t[0] + k];
                c[k] = rest[3 * (size_t)t[3] + k] - rest[3 * (size_t)t[0] + k];
            }
            const double det = a[0] * (b[1] * c[2] - b[2] * c[1]) - a[1] * (b[0] * c[2] - b[2] * c[0]) +
                               a[2] * (b[0] * c[1] - b[1] * c[0]);
            const double mass = (density * std::fabs(det) / 6.0) / 4.0;
            for (int i = 0; i < 4; ++i) m[(size_t)t[i]] += mass;
        }
        return m;
    };
    if (dm->is_set("totalMass") || !(dm->is_set("massDensity") || dm->is_set("vertexMass"))) {
        const double total = dm->get_real(s, "totalMass");
        std::vector<double> m = lumped(1.0);
        double sum = 0.0;
        for (double v : m) sum += v;
        const double density = sum < 1.1920928955078125e-07 ? 1.0 : total / sum;
        for (double& v : m) v *= density;
        return m;
    }
    if (dm->is_set("massDensity")) return lumped(dm->get_real(s, "massDensity"));
    std::vector<double> vm = dm->get_reals(s, "vertexMass");
    if (vm.size() == N) return vm;
    return lumped(1.0);
}

}  // namespace

int Scene::init_host(std::string* err)
{
    if (!root) {
        *err = "scene has no root node";
        return SGB_ERR_INVALID_ARGUMENT;
    }
    // context Data of the root node
    {
        auto it = root->attributes.find("dt");
        if (it != root->attributes.end()) dt = std::strtod(it->second.c_str(), nullptr);
        it = root->attributes.find("gravity");
        if (it != root->attributes.end()) {
            std::istringstream is(it->second);
            for (int k = 0; k < 3; ++k) is >> gravity[k];
        }
    }
    init_tree(*this, root.get());
    // bodies: every node holding an EulerImplicitSolver and a MechanicalObject
    std::vector<Node*> stack{root.get()};
    while (!stack.empty()) {
        Node* n = stack.back();
        stack.pop_back();
        for (auto it = n->children.rbegin(); it != n->children.rend(); ++it) stack.push_back(it->get());
        BaseObject *euler = nullptr, *cg = nullptr, *mo = nullptr, *topo = nullptr, *fem = nullptr, *mass = nullptr;
        BaseObject *pcg = nullptr, *pmfs = nullptr;
        int fem_pos = -1, mass_pos = -1;
        std::vector<BaseObject*> fixed;
        for (size_t i = 0; i < n->objects.size(); ++i) {
            BaseObject* o = n->objects[i].get();
            const std::string& c = o->class_name();
            if (c == "EulerImplicitSolver") euler = o;
            else if (c == "CGLinearSolver") cg = o;
            else if (c == "PCGLinearSolver") pcg = o;
            else if (c == "PreconditionedMatrixFreeSystem") pmfs = o;
            else if (c == "MechanicalObject" && !mo) mo = o;
            else if (c == "TetrahedronSetTopologyContainer" && !topo) topo = o;
            else if (c == "TetrahedronFEMForceField") {
                if (fem) return unsupported(err, "node '" + n->name + "': more than one TetrahedronFEMForceField");
                fem = o;
                fem_pos = (int)i;
            } else if (c == "UniformMass" || c == "DiagonalMass") {
                if (mass) return unsupported(err, "node '" + n->name + "': more than one mass component");
                mass = o;
                mass_pos = (int)i;
            } else if (c == "FixedProjectiveConstraint" || c == "FixedConstraint") {
                fixed.push_back(o);
            }
        }
        if (!euler) continue;
        const std::string where = "node '" + n->name + "': ";
        if (!mo) return unsupported(err, where + "EulerImplicitSolver without a MechanicalObject in the same node");
        if (!cg && !pcg)
            return unsupported(err, where + "EulerImplicitSolver needs a CGLinearSolver or PCGLinearSolver in the same node");
        if (cg && pcg) return unsupported(err, where + "both a CGLinearSolver and a PCGLinearSolver");
        if (!fem) return unsupported(err, where + "no TetrahedronFEMForceField");
        if (!topo) return unsupported(err, where + "no TetrahedronSetTopologyContainer");
        Body b;
        b.node = n;
        b.rest = mo->out_reals["rest_position"];
        const std::vector<double>& x0 = mo->out_reals["position"];
        const std::vector<int>& t = topo->out_ints["tetrahedra"];
        b.tets.assign(t.begin(), t.end());
        const size_t N = b.rest.size() / 3;
        if (N == 0 || b.tets.empty()) return unsupported(err, where + "empty mesh (no positions or no tetrahedra)");
        for (int32_t v : b.tets)
            if (v < 0 || (size_t)v >= N) {
                *err = where + "tetrahedron index out of range";
                return SGB_ERR_INVALID_ARGUMENT;
            }
        // TetrahedronFEMForceField
        const std::string method = fem->get_string("method");
        if (method == "small") b.method = SGB_METHOD_SMALL;
        else if (method == "large") b.method = SGB_METHOD_LARGE;
        else if (method == "polar") b.method = SGB_METHOD_POLAR;
        else if (method == "svd") b.method = SGB_METHOD_SVD;
        else return unsupported(err, where + "TetrahedronFEMForceField method '" + method + "' is not supported");
        if (fem->get_bool(*this, "computeGlobalMatrix") || fem->get_bool(*this, "assembling"))
            return unsupported(err, where + "computeGlobalMatrix=true (assembled matrix) is not supported");
        // updateStiffnessMatrix: polar and svd rebuild J at every addForce
        // (TetrahedronFEMForceField.inl:1063, 1174); small ignores it; the
        // large rebuild (:908-921) writes only some of the entries it builds
        // equal, which the library stores once
        // initialPoints is accepted and, as in the reference, replaced by the
        // MechanicalObject's rest positions when the force field initialises
        // (TetrahedronFEMForceField::reinit, TetrahedronFEMForceField.inl:
        // 1411-1412)
        b.update_stiffness = fem->get_bool(*this, "updateStiffnessMatrix") && b.method != SGB_METHOD_SMALL;
        if (b.update_stiffness && b.method == SGB_METHOD_LARGE)
            return unsupported(err, where + "updateStiffnessMatrix=true with method large (the reference rebuilds "
                                            "only part of the strain-displacement entries, "
                                            "TetrahedronFEMForceField.inl:908-921) is not supported");
        b.plastic_max = fem->get_real(*this, "plasticMaxThreshold");
        b.plastic_yield = fem->get_real(*this, "plasticYieldThreshold");
        b.plastic_creep = fem->get_real(*this, "plasticCreep");
        if (b.plastic_max > 0.0 && b.plastic_yield < 0.0)
            return unsupported(err, where + "plasticYieldThreshold must be >= 0");
        b.von_mises_mode = fem->get_int(*this, "computeVonMisesStress");
        if (b.von_mises_mode < 0 || b.von_mises_mode > 2)
            return unsupported(err, where + "computeVonMisesStress must be 0, 1 or 2");
        if (b.von_mises_mode == 1 && b.method == SGB_METHOD_SMALL)
            return unsupported(err, where + "computeVonMisesStress=1 (corotational strain) needs method large, polar "
                                            "or svd (TetrahedronFEMForceField.inl:1441-1445)");
        b.young = fem->get_reals(*this, "youngModulus");
        b.poisson = fem->get_reals(*this, "poissonRatio");
        const int fallback = precision_of(fem->template_name, SGB_PRECISION_FP64);
        b.precision = precision_override >= 0 ? precision_override : precision_of(mo->template_name, fallback);
        // EulerImplicitSolver + CGLinearSolver
        sgb_scene_params_default(&b.params);
        b.params.trapezoidal_scheme = euler->get_bool(*this, "trapezoidalScheme") ? 1 : 0;
        b.params.dt = dt;
        b.params.first_order = euler->get_bool(*this, "firstOrder") ? 1 : 0;
        b.params.compute_residual = euler->get_bool(*this, "computeResidual") ? 1 : 0;
        // the force field's own rayleighStiffness (BaseForceField.cpp:34): its
        // addDForce factor is kFactorIncludingRayleighDamping
        b.params.ff_rayleigh_stiffness = fem->get_real(*this, "rayleighStiffness");
        b.params.rayleigh_stiffness = euler->get_real(*this, "rayleighStiffness");
        b.params.rayleigh_mass = euler->get_real(*this, "rayleighMass");
        b.params.vdamping = euler->get_real(*this, "vdamping");
        if (cg) {
            b.params.cg_iterations = cg->get_int(*this, "iterations");
            b.params.cg_tolerance = cg->get_real(*this, "tolerance");
            b.params.cg_threshold = cg->get_real(*this, "threshold");
            b.params.warm_start = cg->get_bool(*this, "warmStart") ? 1 : 0;
        } else {
            b.params.linear_solver = SGB_SOLVER_PCG;
            b.params.cg_iterations = pcg->get_int(*this, "iterations");
            b.params.cg_tolerance = pcg->get_real(*this, "tolerance");
            const std::string link = pcg->get_string("preconditioner");
            if (!link.empty() && pcg->get_bool(*this, "use_precond")) {
                BaseObject* pre = resolve_object(n, link);
                if (!pre) return unsupported(err, where + "PCGLinearSolver preconditioner '" + link + "' not found");
                if (pre->class_name() != "JacobiPreconditioner")
                    return unsupported(err, where + "PCGLinearSolver preconditioner " + pre->class_name() +
                                                " is not supported (JacobiPreconditioner is)");
                b.params.preconditioner = SGB_PRECOND_JACOBI;
            }
            int rate = pmfs ? pmfs->get_int(*this, "assemblingRate") : pcg->get_int(*this, "update_step");
            b.params.preconditioner_rate = rate > 1 ? rate : 1;
        }
        for (int k = 0; k < 3; ++k) b.params.gravity[k] = gravity[k];
        // mass
        if (!mass) return unsupported(err, where + "no mass component (UniformMass or DiagonalMass)");
        // the mass's own rayleighMass (BaseMass.cpp:33-34): its addMDx factor
        // is mFactorIncludingRayleighDamping
        b.params.mass_rayleigh_mass = mass->get_real(*this, "rayleighMass");
        // separateGravity moves gravity out of the force into a velocity
        // increment after the position update (UniformMass::addGravityToV,
        // EulerImplicitSolver.cpp:296)
        b.params.separate_gravity = mass->get_bool(*this, "separateGravity") ? 1 : 0;
        if (mass->class_name() == "UniformMass" && !mass->get_ints(*this, "indices").empty())
            return unsupported(err, where + "UniformMass indices (a mass on a subset of the points) is not "
                                            "supported");
        if (mass->class_name() == "UniformMass") {
            // UniformMass::init: totalMass wins over vertexMass when both are
            // set; neither set is an error (UniformMass.inl:233-268)
            if (mass->is_set("totalMass"))
                b.params.vertex_mass = mass->get_real(*this, "totalMass") / (double)N;
            else if (mass->is_set("vertexMass"))
                b.params.vertex_mass = mass->get_real(*this, "vertexMass");
            else
                return unsupported(err, where + "UniformMass needs vertexMass or totalMass");
        } else {
            b.node_masses = diagonal_masses(*this, mass, b.rest, b.tets);
        }
        b.params.mass_first = mass_pos < fem_pos ? 1 : 0;
        // fixed points
        std::set<int> fx;
        int n_project = 0;
        for (BaseObject* f : fixed) {
            if (f->get_bool(*this, "fixAll")) b.params.fix_all = 1;
            if (f->get_bool(*this, "activate_projectVelocity")) n_project++;
            for (int i : f->out_ints["indices"])
                if (i >= 0 && (size_t)i < N) fx.insert(i);
        }
        b.fixed.assign(fx.begin(), fx.end());
        // projectVelocity zeroes the velocity of a component's own indices; the
        // library applies it to every fixed node, so the components must agree
        if (n_project > 0 && n_project < (int)fixed.size())
            return unsupported(err, where + "activate_projectVelocity must be set on every "
                                            "FixedProjectiveConstraint of the node or on none");
        b.params.project_velocity = n_project > 0 ? 1 : 0;
        auto fe = mo->out_reals.find("externalForce");
        if (fe != mo->out_reals.end()) b.external_force = fe->second;
        if (x0.size() == b.rest.size() && x0 != b.rest) mo->out_reals["initial_position"] = x0;
        bodies.push_back(std::move(b));
    }
    return SGB_OK;
}

int Scene::init_device(std::string* err)
{
    for (auto& b : bodies) {
        if (b.scene) continue;
        const int N = (int)(b.rest.size() / 3), E = (int)(b.tets.size() / 4);
        sgb_tfem_t* fem = nullptr;
        int rc = sgb_tfem_create(&fem, N, b.rest.data(), E, b.tets.data(), b.young.data(), (int)b.young.size(),
                                 b.poisson.data(), (int)b.poisson.size(), nullptr, 0, b.method, b.precision);
        if (rc) {
            *err = sgb_last_error();
            return rc;
        }
        if ((b.plastic_max > 0.0 &&
             (rc = sgb_tfem_set_plasticity(fem, b.plastic_max, b.plastic_yield, b.plastic_creep))) ||
            (b.update_stiffness && (rc = sgb_tfem_set_update_stiffness(fem, 1)))) {
            *err = sgb_last_error();
            sgb_tfem_destroy(fem);
            return rc;
        }
        sgb_scene_params p = b.params;
        p.node_masses_host = b.node_masses.empty() ? nullptr : b.node_masses.data();
        p.fixed_host = b.fixed.empty() ? nullptr : b.fixed.data();
        p.n_fixed = (int)b.fixed.size();
        rc = sgb_scene_create(&b.scene, fem, &p);
        if (rc) {
            *err = sgb_last_error();
            sgb_tfem_destroy(fem);
            return rc;
        }
        b.fem = fem;
        if (!b.external_force.empty() && (rc = sgb_scene_set_external_force(b.scene, b.external_force.data()))) {
            *err = sgb_last_error();
            return rc;
        }
        for (auto& o : b.node->objects)
            if (o->class_name() == "MechanicalObject") {
                auto it = o->out_reals.find("initial_position");
                if (it != o->out_reals.end()) {
                    const std::vector<double>& v = o->out_reals["velocity"];
                    if ((rc = sgb_scene_set_state(b.scene, it->second.data(), v.data()))) {
                        *err = sgb_last_error();
                        return rc;
                    }
                }
                break;
            }
    }
    device_ready = true;
    return SGB_OK;
}

static void collect_writers(Node* n, std::vector<WriteState*>& out)
{
    for (auto& o : n->objects)
        if (auto* w = dynamic_cast<WriteState*>(o.get())) out.push_back(w);
    for (auto& c : n->children) collect_writers(c.get(), out);
}

// The reset state of a body's MechanicalObject (MechanicalObject::
// storeResetState, MechanicalObject.inl:1180-1200): its initial positions, and
// its initial velocities when they are not all zero (else zero).
static void reset_state(const Body& b, std::vector<double>& x, std::vector<double>& v)
{
    x = b.rest;
    v.assign(b.rest.size(), 0.0);
    for (auto& o : b.node->objects)
        if (o->class_name() == "MechanicalObject") {
            auto it = o->out_reals.find("initial_position");
            if (it != o->out_reals.end() && it->second.size() == x.size()) x = it->second;
            auto iv = o->out_reals.find("velocity");
            if (iv != o->out_reals.end() && iv->second.size() == v.size()) v = iv->second;
            break;
        }
}

int Scene::reset(std::string* err)
{
    // MechanicalObject::reset (MechanicalObject.inl:1204-1225), the force
    // field's plastic strains (TetrahedronFEMForceField::reset,
    // TetrahedronFEMForceField.inl:1382-1388), WriteState::reset
    // (WriteState.inl:231-238). The solvers keep their own state, as the
    // reference's CGLinearSolver (which has no reset) keeps its time-step count.
    for (auto& b : bodies) {
        if (!b.scene) continue;
        std::vector<double> x, v;
        reset_state(b, x, v);
        int rc = sgb_scene_set_state(b.scene, x.data(), v.data());
        if (!rc && b.plastic_max > 0.0 && b.fem) rc = sgb_tfem_reset_plasticity(b.fem);
        if (rc) {
            *err = sgb_last_error();
            return rc;
        }
    }
    std::vector<WriteState*> writers;
    if (root) collect_writers(root.get(), writers);
    for (WriteState* w : writers) w->rewind();
    time = 0.0;
    return SGB_OK;
}

int Scene::unload()
{
    for (auto& b : bodies) {
        if (b.scene) sgb_scene_destroy(b.scene);
        b.scene = nullptr;
        b.fem = nullptr;
    }
    device_ready = false;
    time = 0.0;
    std::vector<WriteState*> writers;
    if (root) collect_writers(root.get(), writers);
    for (WriteState* w : writers) w->rewind();
    return SGB_OK;
}

int Scene::animate(int n_steps, std::string* err)
{
    if (!device_ready) {
        int rc = init_device(err);
        if (rc) return rc;
    }
    std::vector<WriteState*> writers;
    if (root) collect_writers(root.get(), writers);
    // with state writers the steps go one at a time, each preceded by the
    // writers' animate-begin check; otherwise in one call per body
    const int chunk = writers.empty() ? n_steps : 1;
    for (int done = 0; done < n_steps; done += chunk) {
        for (auto* w : writers) {
            int rc = w->begin_step(*this, time, err);
            if (rc) return rc;
        }
        for (auto& b : bodies) {
            int rc = sgb_scene_step(b.scene, chunk);
            if (rc) {
                *err = sgb_last_error();
                return rc;
            }
        }
        time += dt * chunk;
    }
    return SGB_OK;
}

void register_components(ObjectFactory& f)
{
    const char* mod = "SofaGB300";
    f.register_object("RegularGridTopology", "regular grid of hexahedra", mod, make<RegularGridTopology>());
    f.register_object("Hexa2TetraTopologicalMapping", "6 tetrahedra per hexahedron", mod,
                      make<Hexa2TetraTopologicalMapping>());
    f.register_object("TetrahedronSetTopologyContainer", "tetrahedral topology", mod,
                      make<TetrahedronSetTopologyContainer>());
    f.register_object("TetrahedronSetTopologyModifier", "topology modifier (no effect on a static mesh)", mod,
                      [] { return std::unique_ptr<BaseObject>(new TopologyBookkeeping("TetrahedronSetTopologyModifier")); });
    f.register_object("TetrahedronSetGeometryAlgorithms", "geometry algorithms (no effect on the step)", mod, [] {
        return std::unique_ptr<BaseObject>(new TopologyBookkeeping("TetrahedronSetGeometryAlgorithms"));
    });
    f.register_object("MechanicalObject", "state vectors", mod, make<MechanicalObject>());
    f.register_object("BoxROI", "points inside boxes", mod, make<BoxROI>());
    f.register_object("FixedProjectiveConstraint", "fixed points (projective)", mod,
                      make<FixedProjectiveConstraint>());
    f.register_object("FixedConstraint", "alias of FixedProjectiveConstraint", mod, [] {
        return std::unique_ptr<BaseObject>(new FixedProjectiveConstraint("FixedConstraint"));
    });
    f.register_object("UniformMass", "uniform point mass", mod, make<UniformMass>());
    f.register_object("DiagonalMass", "lumped tetrahedral mass", mod, make<DiagonalMass>());
    f.register_object("TetrahedronFEMForceField", "corotational linear tetrahedral FEM (GB300)", mod,
                      make<TetrahedronFEMForceField>());
    f.register_object("EulerImplicitSolver", "implicit Euler integration", mod, make<EulerImplicitSolver>());
    f.register_object("CGLinearSolver", "matrix-free conjugate gradient", mod, make<CGLinearSolver>());
    f.register_object("PCGLinearSolver", "matrix-free preconditioned conjugate gradient", mod,
                      make<PCGLinearSolver>());
    f.register_object("JacobiPreconditioner", "diagonal (Jacobi) preconditioner", mod,
                      make<JacobiPreconditioner>());
    f.register_object("PreconditionedMatrixFreeSystem", "matrix-free system with an assembled preconditioner", mod,
                      make<PreconditionedMatrixFreeSystem>());
    f.register_object("DefaultAnimationLoop", "animation loop", mod, make<DefaultAnimationLoop>());
    f.register_object("WriteState", "state export (T= / X= / V= lines)", mod, make<WriteState>());
}

}  // namespace scn
}  // namespace sgb
