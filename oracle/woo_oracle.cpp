// CPU oracle for the Woo DEM hot path -- TEST INFRASTRUCTURE ONLY (see woo_oracle.h).
//
// FP64 restatement of the reference's per-step loop, written from the reference
// sources. Every routine cites the reference file:line it restates. Vector,
// matrix and quaternion algebra is written out by hand (the reference uses
// Eigen3); each expression keeps the operand order of the reference expression.
//
// Two modes:
//  * deterministic=0: the reference's OpenMP structure (guided contact loop with
//    per-node atomic force adds, chunked parallel insertion sort). This is the
//    timed CPU baseline.
//  * deterministic=1: contacts kept in (lo id, hi id) order after every collider
//    run and forces applied serially in that order, the reference's
//    Scene.deterministic path (pkg/dem/ContactLoop.cpp:250-257). This is the
//    parity mode the GPU results are compared against.
// In both modes new contacts are oriented (lo id, hi id), which is the
// reference's own (disabled) ordering branch at
// pkg/dem/InsertionSortCollider.cpp:82-85; orientation only changes roundoff.
#include "woo_oracle.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <stdexcept>
#include <string>
#include <unordered_map>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace wo {

static const double Inf = std::numeric_limits<double>::infinity();
static const double PI = 3.14159265358979323846;

struct V3 {
    double x, y, z;
    V3() : x(0), y(0), z(0) {}
    V3(double a, double b, double c) : x(a), y(b), z(c) {}
    double& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
    double operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};
static inline V3 operator+(const V3& a, const V3& b) { return V3(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline V3 operator-(const V3& a, const V3& b) { return V3(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline V3 operator-(const V3& a) { return V3(-a.x, -a.y, -a.z); }
static inline V3 operator*(const V3& a, double s) { return V3(a.x * s, a.y * s, a.z * s); }
static inline V3 operator*(double s, const V3& a) { return V3(s * a.x, s * a.y, s * a.z); }
static inline V3 operator/(const V3& a, double s) { return V3(a.x / s, a.y / s, a.z / s); }
static inline double dot(const V3& a, const V3& b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
static inline double sqn(const V3& a) { return dot(a, a); }
static inline V3 cross(const V3& a, const V3& b) {
    return V3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
static inline bool isZero(const V3& a) { return a.x == 0 && a.y == 0 && a.z == 0; }

// 3x3 matrix, element m[r][c]
struct M3 {
    double m[3][3];
    M3() { std::memset(m, 0, sizeof(m)); }
    static M3 I() { M3 r; r.m[0][0] = r.m[1][1] = r.m[2][2] = 1; return r; }
    V3 col(int c) const { return V3(m[0][c], m[1][c], m[2][c]); }
    void setCol(int c, const V3& v) { m[0][c] = v.x; m[1][c] = v.y; m[2][c] = v.z; }
};
static inline V3 mul(const M3& A, const V3& v) {
    V3 r;
    for (int i = 0; i < 3; i++) r[i] = (A.m[i][0] * v.x + A.m[i][1] * v.y) + A.m[i][2] * v.z;
    return r;
}
// A^T * v: each component is a column of A dotted with v
static inline V3 mulT(const M3& A, const V3& v) {
    V3 r;
    for (int i = 0; i < 3; i++) r[i] = (A.m[0][i] * v.x + A.m[1][i] * v.y) + A.m[2][i] * v.z;
    return r;
}
static inline M3 mmul(const M3& A, const M3& B) {
    M3 r;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) r.m[i][j] = (A.m[i][0] * B.m[0][j] + A.m[i][1] * B.m[1][j]) + A.m[i][2] * B.m[2][j];
    return r;
}
static inline M3 madd(const M3& A, const M3& B) { M3 r; for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) r.m[i][j] = A.m[i][j] + B.m[i][j]; return r; }
static inline M3 msub(const M3& A, const M3& B) { M3 r; for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) r.m[i][j] = A.m[i][j] - B.m[i][j]; return r; }
static inline M3 mscale(const M3& A, double s) { M3 r; for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) r.m[i][j] = A.m[i][j] * s; return r; }
static inline M3 mdiv(const M3& A, double s) { M3 r; for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) r.m[i][j] = A.m[i][j] / s; return r; }
static inline M3 mtr(const M3& A) { M3 r; for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) r.m[i][j] = A.m[j][i]; return r; }
// cofactor-based 3x3 inverse (the closed form Eigen's Matrix3::inverse() evaluates)
static inline double cof(const M3& a, int i, int j) {
    int i1 = (i + 1) % 3, i2 = (i + 2) % 3, j1 = (j + 1) % 3, j2 = (j + 2) % 3;
    return a.m[i1][j1] * a.m[i2][j2] - a.m[i1][j2] * a.m[i2][j1];
}
static inline M3 minv(const M3& a) {
    double c00 = cof(a, 0, 0), c10 = cof(a, 1, 0), c20 = cof(a, 2, 0);
    double det = (c00 * a.m[0][0] + c10 * a.m[1][0]) + c20 * a.m[2][0];
    double invdet = 1.0 / det;
    M3 r;
    r.m[0][0] = c00 * invdet; r.m[0][1] = c10 * invdet; r.m[0][2] = c20 * invdet;
    r.m[1][0] = cof(a, 0, 1) * invdet; r.m[1][1] = cof(a, 1, 1) * invdet; r.m[1][2] = cof(a, 2, 1) * invdet;
    r.m[2][0] = cof(a, 0, 2) * invdet; r.m[2][1] = cof(a, 1, 2) * invdet; r.m[2][2] = cof(a, 2, 2) * invdet;
    return r;
}
// 3x3 determinant expanded along the first row
static inline double mdet(const M3& a) {
    return (a.m[0][0] * (a.m[1][1] * a.m[2][2] - a.m[1][2] * a.m[2][1]) - a.m[0][1] * (a.m[1][0] * a.m[2][2] - a.m[1][2] * a.m[2][0])) +
           a.m[0][2] * (a.m[1][0] * a.m[2][1] - a.m[1][1] * a.m[2][0]);
}
// dual vector of a skew matrix, lib/base/Math.hpp:222-227
static inline bool isIdentity(const M3& a) {
    for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) if (a.m[i][j] != (i == j ? 1. : 0.)) return false;
    return true;
}
static inline V3 leviCivita(const M3& m) { return V3(m.m[1][2] - m.m[2][1], m.m[2][0] - m.m[0][2], m.m[0][1] - m.m[1][0]); }

struct Q { double w, x, y, z; };
static inline Q qmul(const Q& a, const Q& b) {
    Q r;
    r.w = ((a.w * b.w - a.x * b.x) - a.y * b.y) - a.z * b.z;
    r.x = ((a.w * b.x + a.x * b.w) + a.y * b.z) - a.z * b.y;
    r.y = ((a.w * b.y + a.y * b.w) + a.z * b.x) - a.x * b.z;
    r.z = ((a.w * b.z + a.z * b.w) + a.x * b.y) - a.y * b.x;
    return r;
}
static inline void qnormalize(Q& q) {
    double n = std::sqrt(((q.x * q.x + q.y * q.y) + q.z * q.z) + q.w * q.w);
    q.w = q.w / n; q.x = q.x / n; q.y = q.y / n; q.z = q.z / n;
}
// quaternion from rotation matrix (Shepperd's method, as used for Quaternionr(Matrix3r)),
// the L6Geom node orientation, pkg/dem/L6Geom.cpp:69,216
static inline Q quatFromMat(const M3& m) {
    Q q;
    double t = (m.m[0][0] + m.m[1][1]) + m.m[2][2];
    if (t > 0) {
        t = std::sqrt(t + 1.0);
        q.w = 0.5 * t;
        t = 0.5 / t;
        q.x = (m.m[2][1] - m.m[1][2]) * t;
        q.y = (m.m[0][2] - m.m[2][0]) * t;
        q.z = (m.m[1][0] - m.m[0][1]) * t;
    } else {
        int i = 0;
        if (m.m[1][1] > m.m[0][0]) i = 1;
        if (m.m[2][2] > m.m[i][i]) i = 2;
        int j = (i + 1) % 3, k = (j + 1) % 3;
        t = std::sqrt(((m.m[i][i] - m.m[j][j]) - m.m[k][k]) + 1.0);
        double c[3];
        c[i] = 0.5 * t;
        t = 0.5 / t;
        q.w = (m.m[k][j] - m.m[j][k]) * t;
        c[j] = (m.m[j][i] + m.m[i][j]) * t;
        c[k] = (m.m[k][i] + m.m[i][k]) * t;
        q.x = c[0]; q.y = c[1]; q.z = c[2];
    }
    return q;
}
// rotate vector by quaternion: v + w*(2 q x v) + q x (2 q x v)
static inline V3 qrot(const Q& q, const V3& v) {
    V3 qv(q.x, q.y, q.z);
    V3 uv = cross(qv, v);
    uv = uv + uv;
    return (v + q.w * uv) + cross(qv, uv);
}

enum { SH_SPHERE = 0, SH_WALL = 1, SH_FACET = 2 };
// DemData flag bits, pkg/dem/Particle.hpp:179-186
enum { DOF_X = 1, DOF_Y = 2, DOF_Z = 4, DOF_RX = 8, DOF_RY = 16, DOF_RZ = 32, DOF_ALL = 63, DOF_RXRYRZ = 56,
       CLUMP_CLUMPED = 64, CLUMP_CLUMP = 128, ENERGY_SKIP = 256, GRAVITY_SKIP = 512, DAMPING_SKIP = 2048 };
enum { HOMO_NONE = 0, HOMO_POS = 1, HOMO_VEL = 2, HOMO_VEL_2ND = 3, HOMO_GRADV2 = 4 };
// Scene.energy entries (EnergyTracker), in the order of wo_get_energy
enum { EN_KINETIC, EN_KINTRANS, EN_KINROT, EN_GRAV, EN_DAMP, EN_ELAST, EN_PLAST, EN_BROKEN, EN_VISCN, EN_VISCT, EN_GRADV, EN_N };

struct Node {
    V3 pos; Q ori;
    V3 vel, angVel, force, torque, inertia;
    double mass; uint32_t flags;
};
struct Material { double density, young, tanPhi, ktDivKn; };
struct Particle {
    int shape; int nodes[3]; double radius; int axis, sense; double halfThick; V3 fakeVel; int mat; uint32_t mask;
    bool hasBound; V3 mn, mx; V3 lastPos[3]; double maxD2;
    int nNodes() const { return shape == SH_FACET ? 3 : 1; }
};
struct Contact {
    int pA, pB; int cellDist[3]; int stepCreated; double minDist00Sq; bool geom, phys;
    // L6Geom (pkg/dem/L6Geom.hpp:14-22) with its node (pos, ori)
    M3 trsf; V3 cpos; Q cori; double uN; double lens[2]; double contA; V3 lvel, langVel;
    // FrictPhys / HertzPhys (pkg/dem/FrictMat.hpp:30-41, pkg/dem/Hertz.hpp:5-21)
    double kn, kt, tanPhi; V3 force, torque;
    double K, R, kt0, alpha_sqrtMK, gamma, alpha;
    // energies added by the law in the current step: elast, plast, broken, viscN, viscT, and the
    // number of elast and broken additions
    double en[5]; int enN[2];
    size_t linIx;
    bool isReal() const { return geom && phys; }
    void reset() { geom = false; phys = false; }
};
static inline uint64_t ckey(int a, int b) { int lo = std::min(a, b), hi = std::max(a, b); return ((uint64_t)(uint32_t)lo << 32) | (uint32_t)hi; }

// periodic cell, core/Cell.hpp:22-187, core/Cell.cpp:28-120
struct Cell {
    M3 trsf, hSize, pprevHsize, gradV, nextGradV, W; V3 spinVec; int homoDeform;
    M3 invTrsf, trsfInc, shearTrsf, unshearTrsf; V3 size, cosv; bool hasShear;
    Cell() : trsf(M3::I()), hSize(M3::I()), pprevHsize(M3::I()), homoDeform(HOMO_GRADV2), invTrsf(M3::I()) {}
    void integrateAndUpdate(double dt) {
        trsfInc = mscale(gradV, dt);
        trsf = madd(trsf, mmul(trsfInc, trsf));
        invTrsf = minv(trsf);
        M3 prevHsize = hSize;
        if (homoDeform == HOMO_GRADV2) {
            M3 a = minv(msub(M3::I(), mdiv(mscale(gradV, dt), 2.)));
            M3 b = madd(M3::I(), mdiv(mscale(gradV, dt), 2.));
            hSize = mmul(mmul(a, b), hSize);
        } else hSize = madd(hSize, mmul(trsfInc, hSize));
        pprevHsize = mscale(madd(prevHsize, hSize), .5);
        if (mdet(hSize) == 0) throw std::runtime_error("Cell is degenerate (zero volume).");
        M3 Hnorm;
        for (int i = 0; i < 3; i++) {
            V3 base = hSize.col(i);
            size[i] = std::sqrt(sqn(base));
            base = base / size[i];
            Hnorm.setCol(i, base);
        }
        for (int i = 0; i < 3; i++) {
            int i1 = (i + 1) % 3, i2 = (i + 2) % 3;
            cosv[i] = sqn(cross(Hnorm.col(i1), Hnorm.col(i2)));
        }
        shearTrsf = Hnorm;
        unshearTrsf = minv(shearTrsf);
        hasShear = (hSize.m[0][1] != 0 || hSize.m[0][2] != 0 || hSize.m[1][0] != 0 || hSize.m[1][2] != 0 || hSize.m[2][0] != 0 || hSize.m[2][1] != 0);
    }
    void setNextGradV() {
        gradV = nextGradV;
        W = mscale(msub(gradV, mtr(gradV)), .5);
        spinVec = .5 * leviCivita(W);
    }
    V3 intrShiftPos(const int cd[3]) const { return mul(hSize, V3(cd[0], cd[1], cd[2])); }
    V3 intrShiftVel(const int cd[3]) const {
        V3 c(cd[0], cd[1], cd[2]);
        switch (homoDeform) {
            case HOMO_VEL: case HOMO_VEL_2ND: return mul(mmul(gradV, hSize), c);
            case HOMO_GRADV2: return mul(mmul(gradV, pprevHsize), c);
            default: return V3();
        }
    }
    V3 pprevFluctVel(const V3& currPos, const V3& pprevVel, double dt) const {
        switch (homoDeform) {
            case HOMO_NONE: case HOMO_POS: return pprevVel;
            case HOMO_VEL: case HOMO_VEL_2ND: return pprevVel - mul(gradV, currPos);
            default: return pprevVel - mul(gradV, currPos - (dt / 2) * pprevVel);
        }
    }
    V3 pprevFluctAngVel(const V3& a) const { return homoDeform == HOMO_GRADV2 ? a - spinVec : a; }
    V3 shearAlignedExtents(const V3& perp) const {
        if (!hasShear) return perp;
        V3 ret = perp;
        for (int ax = 0; ax < 3; ax++) {
            int ax1 = (ax + 1) % 3, ax2 = (ax + 2) % 3;
            ret[ax1] += .5 * perp[ax1] * (1 / cosv[ax] - 1);
            ret[ax2] += .5 * perp[ax2] * (1 / cosv[ax] - 1);
        }
        return ret;
    }
    V3 unshearPt(const V3& p) const { return mul(unshearTrsf, p); }
};

struct Bounds {
    double coord; int id; int period; bool hasBB, isMin, isInf;
    // pkg/dem/InsertionSortCollider.hpp:130-138
    bool lt(const Bounds& b) const { if (id == b.id && coord == b.coord) return isMin; return coord < b.coord; }
    bool gt(const Bounds& b) const { if (id == b.id && coord == b.coord) return !isMin; return coord > b.coord; }
};
struct VecBounds {
    int axis = -1; std::vector<Bounds> vec; double cellDim = 0; long size = 0; long loIdx = 0;
    long norm(long i) const { if (i < 0) i += size; return i % size; }
    Bounds& operator[](long i) { return vec[i]; }
};

struct Scene {
    wo_config cfg;
    std::string err;
    std::vector<Node> nodes;
    std::vector<Particle> par;
    std::vector<Material> mats;
    Cell cell;
    long step = 0; double time = 0;
    int nThreads = 1;
    // collider state (pkg/dem/InsertionSortCollider.hpp:147-175)
    VecBounds BB[3];
    std::vector<double> minima, maxima;
    bool colliderPeriodic = false;
    long nFullRuns = 0;
    double verletDist = 0;
    bool verletInit = false;
    std::vector<std::vector<std::pair<int, int>>> makeLater;  // (id1,id2) per thread
    std::vector<std::vector<int>> makeLaterPeri;              // periods, 3 per entry
    std::vector<std::vector<Contact*>> removeLater;
    // contacts (pkg/dem/ContactContainer.hpp)
    std::vector<Contact*> linView;
    std::unordered_map<uint64_t, Contact*> cmap;
    std::vector<std::vector<Contact*>> pending;
    M3 stress;
    double sqrt5, viscAlphaConst; bool viscOn;
    // Scene.energy and whether each entry exists
    double energy[EN_N] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
    int ecreated[EN_N] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
    // ContactLoop.prevStress and prevVol (ContactLoop.hpp:119-123)
    M3 prevStress; double prevVol = std::numeric_limits<double>::quiet_NaN();

    ~Scene() { for (auto* c : linView) delete c; }

    Contact* find(int a, int b) const { auto it = cmap.find(ckey(a, b)); return it == cmap.end() ? nullptr : it->second; }
    // ContactContainer::addMaybe_fast, pkg/dem/ContactContainer.cpp:51-58
    void addMaybe_fast(Contact* c) {
        uint64_t k = ckey(c->pA, c->pB);
        if (cmap.count(k)) { delete c; return; }
        cmap[k] = c; linView.push_back(c); c->linIx = linView.size() - 1;
    }
    // ContactContainer::linView_remove, pkg/dem/ContactContainer.cpp:69-80
    void linView_remove(size_t ix) {
        if (ix < linView.size() - 1) { linView[ix] = linView.back(); linView[ix]->linIx = ix; }
        linView.resize(linView.size() - 1);
    }
    // ContactContainer::removeMaybe_fast / remove, pkg/dem/ContactContainer.cpp:60-67,82-137
    void removeMaybe_fast(Contact* c) {
        auto it = cmap.find(ckey(c->pA, c->pB));
        if (it == cmap.end() || it->second != c) return;
        cmap.erase(it);
        linView_remove(c->linIx);
        delete c;
    }
    int tid() const {
#ifdef _OPENMP
        return omp_get_thread_num();
#else
        return 0;
#endif
    }

    // Collider::mayCollide, pkg/dem/Collision.cpp:19-41 (no clumps here: nodes are never shared
    // between a sphere and anything else in the supported shapes, so the node test reduces to ids)
    bool mayCollide(int a, int b) const {
        if (a == b) return false;
        const Particle &A = par[a], &B = par[b];
        if (!(A.mask & B.mask)) return false;
        if ((A.mask & B.mask & cfg.lone_mask) != 0) return false;
        for (int i = 0; i < A.nNodes(); i++)
            for (int j = 0; j < B.nNodes(); j++)
                if (A.nodes[i] == B.nodes[j]) return false;
        return true;
    }

    // ------------------------------------------------------------ Bo1 functors
    // Bo1_Sphere_Aabb::go/goGeneric pkg/dem/Sphere.cpp:50-79; Bo1_Wall_Aabb pkg/dem/Wall.cpp:24-33;
    // Bo1_Facet_Aabb pkg/dem/Facet.cpp:177-200
    void boundFunctor(Particle& p) {
        p.hasBound = true;
        if (p.shape == SH_SPHERE) {
            double f = (cfg.bo1_sphere_dist_factor > 0 ? cfg.bo1_sphere_dist_factor : 1.) * p.radius;
            V3 h(f, f, f);
            const V3& pos = nodes[p.nodes[0]].pos;
            if (!cfg.periodic) { p.mn = pos - h; p.mx = pos + h; return; }
            h = cell.shearAlignedExtents(h);
            p.mn = cell.unshearPt(pos) - h; p.mx = cell.unshearPt(pos) + h;
        } else if (p.shape == SH_WALL) {
            if (cfg.periodic && cell.hasShear) throw std::logic_error("Walls not supported in skewed (Scene.cell.trsf is not diagonal) periodic boundary conditions.");
            p.mn = V3(-Inf, -Inf, -Inf); p.mx = V3(Inf, Inf, Inf);
            p.mn[p.axis] = p.mx[p.axis] = nodes[p.nodes[0]].pos[p.axis];
        } else {
            V3 h(p.halfThick, p.halfThick, p.halfThick);
            V3 v0 = cfg.periodic ? cell.unshearPt(nodes[p.nodes[0]].pos) : nodes[p.nodes[0]].pos;
            p.mn = v0 - h; p.mx = v0 + h;
            for (int i = 1; i < 3; i++) {
                V3 v = cfg.periodic ? cell.unshearPt(nodes[p.nodes[i]].pos) : nodes[p.nodes[i]].pos;
                V3 a = v - h, b = v + h;
                for (int k = 0; k < 3; k++) { p.mn[k] = std::min(p.mn[k], a[k]); p.mx[k] = std::max(p.mx[k], b[k]); }
            }
        }
    }

    // InsertionSortCollider::updateBboxes_doFullRun, pkg/dem/InsertionSortCollider.cpp:281-417
    bool updateBboxes_doFullRun() {
        if (!verletInit) {
            verletInit = true;
            verletDist = cfg.verlet_dist;
            if (verletDist < 0) {
                double minR = Inf;
                for (auto& p : par) if (p.shape == SH_SPHERE) minR = std::min(p.radius, minR);
                verletDist = std::isinf(minR) ? 0 : std::abs(verletDist) * minR;
            }
        }
        bool recompute = false;
        if (verletDist == 0) recompute = true;
        else {
            for (auto& p : par) {
                if (!p.hasBound) { recompute = true; break; }
                if (std::isnan(std::max(std::max(p.mn.x, p.mn.y), p.mn.z)) || std::isnan(std::max(std::max(p.mx.x, p.mx.y), p.mx.z))) { recompute = true; break; }
                double d2 = 0;
                for (int i = 0; i < p.nNodes(); i++) d2 = std::max(d2, sqn(p.lastPos[i] - nodes[p.nodes[i]].pos));
                if (d2 + 0. > p.maxD2) { recompute = true; break; }
            }
        }
        if (!recompute) return false;
        long n = (long)par.size();
        std::string ex;
#pragma omp parallel for num_threads(nThreads)
        for (long i = 0; i < n; i++) {
            try {
                Particle& p = par[i];
                boundFunctor(p);
                for (int k = 0; k < p.nNodes(); k++) p.lastPos[k] = nodes[p.nodes[k]].pos;
                p.maxD2 = verletDist * verletDist;
                if (verletDist > 0) {
                    V3 vd(verletDist, verletDist, verletDist);
                    p.mx = p.mx + vd; p.mn = p.mn - vd;
                }
            } catch (std::exception& e) {
#pragma omp critical
                ex = e.what();
            }
        }
        if (!ex.empty()) throw std::runtime_error(ex);
        return true;
    }

    // InsertionSortCollider::spatialOverlap, pkg/dem/InsertionSortCollider.cpp:52-58
    bool spatialOverlap(int id1, int id2) const {
        return (minima[3 * id1 + 0] <= maxima[3 * id2 + 0]) && (maxima[3 * id1 + 0] >= minima[3 * id2 + 0]) &&
               (minima[3 * id1 + 1] <= maxima[3 * id2 + 1]) && (maxima[3 * id1 + 1] >= minima[3 * id2 + 1]) &&
               (minima[3 * id1 + 2] <= maxima[3 * id2 + 2]) && (maxima[3 * id1 + 2] >= minima[3 * id2 + 2]);
    }
    // cellWrap / cellWrapRel, pkg/dem/InsertionSortCollider.cpp:650-660
    static double cellWrap(double x, double x0, double x1, int& period) {
        double xNorm = (x - x0) / (x1 - x0);
        period = (int)std::floor(xNorm);
        return x0 + (xNorm - period) * (x1 - x0);
    }
    static double cellWrapRel(double x, double x0, double x1) {
        double xNorm = (x - x0) / (x1 - x0);
        return (xNorm - std::floor(xNorm)) * (x1 - x0);
    }
    // InsertionSortCollider::spatialOverlapPeri, pkg/dem/InsertionSortCollider.cpp:903-957
    bool spatialOverlapPeri(int id1, int id2, int periods[3]) const {
        for (int axis = 0; axis < 3; axis++) {
            double dim = cell.size[axis];
            double m1 = minima[3 * id1 + axis], m2 = minima[3 * id2 + axis];
            if (std::isinf(m1) || std::isinf(m2)) { periods[axis] = 0; continue; }
            double wMn = (cellWrapRel(m1, m2, m2 + dim) < cellWrapRel(m2, m1, m1 + dim)) ? m2 : m1;
            int pmn1, pmx1, pmn2, pmx2;
            double mn1 = cellWrap(minima[3 * id1 + axis], wMn, wMn + dim, pmn1), mx1 = cellWrap(maxima[3 * id1 + axis], wMn, wMn + dim, pmx1);
            double mn2 = cellWrap(minima[3 * id2 + axis], wMn, wMn + dim, pmn2), mx2 = cellWrap(maxima[3 * id2 + axis], wMn, wMn + dim, pmx2);
            if ((pmn1 != pmx1) || (pmn2 != pmx2))
                throw std::runtime_error("InsertionSortCollider: Particle larger than half of the cell size encountered.");
            periods[axis] = (int)(pmn1 - pmn2);
            if (!(mn1 <= mx2 && mx1 >= mn2)) return false;
        }
        return true;
    }
    bool shouldBeRemoved(const Contact* C) const {
        if (!colliderPeriodic) return !spatialOverlap(C->pA, C->pB);
        int p[3]; return !spatialOverlapPeri(C->pA, C->pB, p);
    }
    void makeContactLater(int id1, int id2, const int* periods) {
        int t = tid();
        makeLater[t].push_back(std::make_pair(id1, id2));
        for (int k = 0; k < 3; k++) makeLaterPeri[t].push_back(periods ? periods[k] : 0);
    }
    // InsertionSortCollider::handleBoundInversion, pkg/dem/InsertionSortCollider.cpp:63-98
    void handleBoundInversion(int id1, int id2, bool separating) {
        bool overlap = separating ? false : spatialOverlap(id1, id2);
        Contact* C = find(id1, id2);
        bool hasCon = C != nullptr;
        if (!overlap && !hasCon) return;
        if (overlap && hasCon) return;
        if (overlap) { if (!mayCollide(id1, id2)) return; makeContactLater(id1, id2, nullptr); return; }
        if (!C->isReal()) removeLater[tid()].push_back(C);
    }
    // InsertionSortCollider::handleBoundInversionPeri, pkg/dem/InsertionSortCollider.cpp:836-874
    void handleBoundInversionPeri(int id1, int id2, bool separating) {
        int periods[3] = {0, 0, 0};
        bool overlap = separating ? false : spatialOverlapPeri(id1, id2, periods);
        Contact* C = find(id1, id2);
        bool hasCon = C != nullptr;
        if (!overlap && !hasCon) return;
        if (overlap && hasCon) return;
        if (overlap) { if (!mayCollide(id1, id2)) return; makeContactLater(id1, id2, periods); return; }
        if (!C->isReal()) removeLater[tid()].push_back(C);
    }
    // InsertionSortCollider::insertionSort_part, pkg/dem/InsertionSortCollider.cpp:162-196
    void insertionSort_part(VecBounds& v, bool doCollide, long iBegin, long iEnd, long iStart) {
        const bool earlyStop = (iBegin != iStart);
        for (long i = std::max(iStart, iBegin + 1); i < iEnd; i++) {
            if (!(v[i - 1].gt(v[i]))) { if (earlyStop) return; continue; }
            const Bounds viInit = v[i]; long j = i - 1;
            const bool viInitBB = viInit.hasBB, viInitIsMin = viInit.isMin;
            while (j >= iBegin && v[j].gt(viInit)) {
                v[j + 1] = v[j];
                if (viInitIsMin != v[j].isMin && doCollide && viInitBB && v[j].hasBB && (viInit.id != v[j].id))
                    handleBoundInversion(viInit.id, v[j].id, !viInitIsMin);
                j--;
            }
            v[j + 1] = viInit;
        }
    }
    // InsertionSortCollider::insertionSort (OpenMP chunked variant), pkg/dem/InsertionSortCollider.cpp:100-159
    void insertionSort(VecBounds& v, bool doCollide) {
        int TH = nThreads;
        long chunks_per_core = 1, min_per_core = 2 * 1000, max_per_core = 0;  // ompTuneSort default (1,1000,0)
        long chunks = TH * std::max(1L, chunks_per_core);
        if (min_per_core > 0 && (long)(v.size / chunks) < min_per_core) chunks = TH * (long)std::ceil(std::max(1L, v.size / min_per_core) * 1. / TH);
        else if (max_per_core > 0 && (long)(v.size / chunks) > max_per_core) chunks = TH * (long)std::ceil(std::max(1L, v.size / max_per_core) * 1. / TH);
        long chunkSize = v.size / chunks;
        if (chunks == 1 || chunkSize < 100) { insertionSort_part(v, doCollide, 0, v.size, 0); return; }
        std::vector<long> splits0(chunks + 1), splits1(chunks);
        for (long i = 0; i < chunks; i++) { splits0[i] = i * chunkSize; splits1[i] = i * chunkSize + chunkSize / 2; }
        splits0[chunks] = v.size;
        bool isOk = false;
        for (long pass = 0; !isOk; pass++) {
            bool even = ((pass % 2) == 0);
            const std::vector<long>& s(even ? splits0 : splits1);
            long nch = even ? chunks : chunks - 1;
#pragma omp parallel for schedule(static) num_threads(nThreads)
            for (long chunk = 0; chunk < nch; chunk++) {
                long start = (pass == 0 ? s[chunk] : (even ? splits1[chunk] : splits0[chunk + 1]));
                insertionSort_part(v, doCollide, s[chunk], s[chunk + 1], start);
            }
            isOk = true;
            for (long chunk = (even ? 1 : 0); chunk < chunks; chunk++) {
                if (v[s[chunk] - 1].gt(v[s[chunk]])) { isOk = false; break; }
            }
        }
    }
    // InsertionSortCollider::insertionSortPeri_part (serial form), pkg/dem/InsertionSortCollider.cpp:718-791
    void insertionSortPeri(VecBounds& v, bool doCollide) {
        if (v.size == 0) return;
        long& loIdx = v.loIdx;
        for (long _i = 0; _i < v.size; _i++) {
            const long i = v.norm(_i);
            const long i_1 = v.norm(i - 1);
            if (i == loIdx && v[i].coord < 0) { v[i].period -= 1; v[i].coord += v.cellDim; loIdx = v.norm(loIdx + 1); }
            const double iCmpCoord = v[i].coord + (i == loIdx ? v.cellDim : 0);
            if (v[i_1].coord <= iCmpCoord) continue;
            long j = i_1; Bounds vi = v[i];
            const bool viHasBB = vi.hasBB, viIsMin = vi.isMin, viIsInf = vi.isInf;
            while (v[j].coord > vi.coord + (v.norm(j + 1) == loIdx ? v.cellDim : 0)) {
                long j1 = v.norm(j + 1);
                Bounds& vNew = v[j1];
                vNew = v[j];
                if (j == loIdx && vi.coord < 0) { vi.period -= 1; vi.coord += v.cellDim; loIdx = v.norm(loIdx + 1); }
                else if (j1 == loIdx) { vNew.period += 1; vNew.coord -= v.cellDim; loIdx = v.norm(loIdx - 1); }
                if (viIsMin != v[j].isMin && doCollide && viHasBB && v[j].hasBB) {
                    if (vi.id != vNew.id) handleBoundInversionPeri(vi.id, vNew.id, (!viIsMin && !viIsInf && !v[j].isInf));
                }
                j = v.norm(j - 1);
            }
            v[v.norm(j + 1)] = vi;
        }
    }
    // ContactContainer::removePending, pkg/dem/ContactContainer.hpp:78-93
    void removePending() {
        for (auto& pl : pending) {
            for (Contact* c : pl) if (shouldBeRemoved(c)) removeMaybe_fast(c);
            pl.clear();
        }
    }
    // InsertionSortCollider::makeRemoveContactLater_process, pkg/dem/InsertionSortCollider.cpp:20-48
    void makeRemoveContactLater_process() {
        for (auto& rl : removeLater) { for (Contact* c : rl) removeMaybe_fast(c); rl.clear(); }
        for (size_t t = 0; t < makeLater.size(); t++) {
            for (size_t k = 0; k < makeLater[t].size(); k++) {
                Contact* C = new Contact();
                int id1 = makeLater[t][k].first, id2 = makeLater[t][k].second;
                const int* pr = &makeLaterPeri[t][3 * k];
                // canonical orientation (lo id first); periods belong to (id1,id2) and flip with the order
                int sgn = 1;
                if (id1 > id2) { std::swap(id1, id2); sgn = -1; }
                C->pA = id1; C->pB = id2;
                for (int a = 0; a < 3; a++) C->cellDist[a] = sgn * pr[a];
                C->stepCreated = (int)step; C->minDist00Sq = -1; C->geom = C->phys = false;
                addMaybe_fast(C);
            }
            makeLater[t].clear(); makeLaterPeri[t].clear();
        }
    }
    // InsertionSortCollider::run, pkg/dem/InsertionSortCollider.cpp:445-646 (+ prologue_doFullRun :419-443)
    void colliderRun(bool forceFull = false) {
        bool fullRun = forceFull;
        long nPar = (long)par.size();
        if ((long)BB[0].size != 2 * nPar) fullRun = true;
        if (cfg.periodic != (int)colliderPeriodic) { for (int i = 0; i < 3; i++) BB[i].vec.clear(), BB[i].size = 0; colliderPeriodic = cfg.periodic; fullRun = true; }
        bool runBboxes = updateBboxes_doFullRun();
        if (runBboxes) fullRun = true;
        if (!fullRun) { removePending(); return; }
        nFullRuns++;
        bool doInitSort = false;
        if (BB[0].size != 2 * nPar) {
            if (2 * nPar < BB[0].size) { for (int i = 0; i < 3; i++) { BB[i].vec.clear(); BB[i].size = 0; } }
            else if (2 * nPar - BB[0].size > 200 || BB[0].size == 0) doInitSort = true;
            for (int i = 0; i < 3; i++) {
                BB[i].axis = i;
                for (long id = (long)BB[i].vec.size() / 2; id < nPar; id++) {
                    Bounds a{0, (int)id, 0, false, true, false}, b{0, (int)id, 0, false, false, false};
                    BB[i].vec.push_back(a); BB[i].vec.push_back(b);
                }
                BB[i].size = (long)BB[i].vec.size();
            }
        }
        if ((long)minima.size() != 3 * nPar) { minima.resize(3 * nPar); maxima.resize(3 * nPar); }
        if (colliderPeriodic) for (int i = 0; i < 3; i++) BB[i].cellDim = cell.size[i];
        long n2 = 2 * nPar;
#pragma omp parallel for schedule(static) num_threads(nThreads)
        for (long i = 0; i < n2; i++) {
            for (int j = 0; j < 3; j++) {
                VecBounds& BBj = BB[j];
                Bounds& b = BBj[i];
                const Particle& p = par[b.id];
                b.hasBB = p.hasBound;
                b.coord = (b.hasBB ? (b.isMin ? p.mn[j] : p.mx[j]) : nodes[p.nodes[0]].pos[j]) - (colliderPeriodic ? BBj.cellDim * b.period : 0.);
                b.isInf = false;
                if (colliderPeriodic && std::isinf(b.coord)) { b.period = (b.coord < 0 ? 0 : 1); b.coord = 0.; b.isInf = true; }
                if (doInitSort && colliderPeriodic) { if (!b.isInf) b.coord = cellWrap(b.coord, 0, BBj.cellDim, b.period); }
            }
        }
        for (long id = 0; id < nPar; id++) {
            const Particle& p = par[id];
            for (int k = 0; k < 3; k++) { minima[3 * id + k] = p.mn[k]; maxima[3 * id + k] = p.mx[k]; }
        }
        removePending();
        if (!doInitSort) {
            if (!colliderPeriodic) for (int i = 0; i < 3; i++) insertionSort(BB[i], true);
            else for (int i = 0; i < 3; i++) insertionSortPeri(BB[i], true);
        } else {
            for (int i = 0; i < 3; i++) {
                BB[i].loIdx = 0;
                std::sort(BB[i].vec.begin(), BB[i].vec.end(), [](const Bounds& a, const Bounds& b) { return a.lt(b); });
            }
            // The reference sweeps serially (InsertionSortCollider.cpp:605-632); the sweep only
            // fills the contact container, and the pairs do not depend on the order in which it
            // visits the bounds (the deterministic mode re-sorts the container by key after every
            // collider run), so it is split over the threads here: serially it takes minutes at a
            // million spheres, where one sort-axis slab holds thousands of boxes.
            VecBounds& V = BB[cfg.sort_axis];
            if (!colliderPeriodic) {
#pragma omp parallel for schedule(dynamic, 256) num_threads(nThreads)
                for (long i = 0; i < n2; i++) {
                    if (!(V[i].isMin && V[i].hasBB)) continue;
                    const int iid = V[i].id;
                    for (long j = i + 1; j < n2 && V[j].id != iid; j++) {
                        if (!V[j].isMin) continue;
                        handleBoundInversion(iid, V[j].id, false);
                    }
                }
            } else {
                bool loop = false;
#pragma omp parallel for schedule(dynamic, 256) num_threads(nThreads)
                for (long i = 0; i < n2; i++) {
                    if (!(V[i].isMin && V[i].hasBB)) continue;
                    const int iid = V[i].id;
                    long cnt = 0;
                    for (long j = V.norm(i + 1); V[j].id != iid; j = V.norm(j + 1)) {
                        if (!V[j].isMin) continue;
                        handleBoundInversionPeri(iid, V[j].id, false);
                        if (cnt++ > 2 * nPar) {
#pragma omp atomic write
                            loop = true;
                            break;
                        }
                    }
                }
                if (loop) throw std::logic_error("Uninterrupted loop in the initial sort?");
            }
        }
        makeRemoveContactLater_process();
        if (cfg.deterministic) {
            std::sort(linView.begin(), linView.end(), [](const Contact* a, const Contact* b) { return ckey(a->pA, a->pB) < ckey(b->pA, b->pB); });
            for (size_t i = 0; i < linView.size(); i++) linView[i]->linIx = i;
        }
    }

    // ------------------------------------------------------------ L6Geom
    // L6Geom::setInitialLocalCoords, pkg/dem/L6Geom.cpp:27-38
    static void setInitialLocalCoords(Contact* C, const V3& locX) {
        V3 ref = (std::abs(locX.y) < std::abs(locX.z)) ? V3(0, 1, 0) : V3(0, 0, 1);
        V3 locY = cross(locX, ref);
        locY = locY - locX * dot(locY, locX);
        { double z = sqn(locY); if (z > 0) locY = locY / std::sqrt(z); }
        V3 locZ = cross(locX, locY);
        C->trsf.setCol(0, locX); C->trsf.setCol(1, locY); C->trsf.setCol(2, locZ);
    }
    // Cg2_Any_Any_L6Geom__Base::handleSpheresLikeContact, pkg/dem/L6Geom.cpp:51-217
    void handleSpheresLikeContact(Contact* C, const V3& pos1, const V3& vel1, const V3& angVel1, const V3& pos2, const V3& vel2,
                                  const V3& angVel2, const V3& normal, const V3& contPt, double uN, double r1, double r2) {
        const double dt = cfg.dt;
        const int approxMask = cfg.approx_mask;
        if (!C->geom) {
            C->geom = true;
            setInitialLocalCoords(C, normal);
            C->uN = uN;
            C->lens[0] = std::abs(r1) + uN / 2; C->lens[1] = std::abs(r2) + uN / 2;
            if (C->lens[0] < 0) C->lens[0] = C->lens[1];
            if (C->lens[1] < 0) C->lens[1] = C->lens[0];
            double rr = (r1 > 0 && r2 > 0) ? std::min(r1, r2) : (r1 > 0 ? r1 : r2);
            C->contA = PI * (rr * rr);
            C->lvel = V3(); C->langVel = V3();
            C->cpos = contPt;
            C->cori = quatFromMat(C->trsf);
            return;
        }
        const V3 currNormal = normal; const V3 prevNormal = C->trsf.col(0);
        const V3 prevContPt = C->cpos;
        V3 shiftVel2 = cfg.periodic ? cell.intrShiftVel(C->cellDist) : V3();
        V3 normRotVec = cross(prevNormal, currNormal);
        V3 midNormal = (approxMask & 1) ? prevNormal : .5 * (prevNormal + currNormal);
        if (std::sqrt(sqn(midNormal)) == 0) midNormal = currNormal;
        else if (!(approxMask & 2) && !(approxMask & 1)) { double z = sqn(midNormal); if (z > 0) midNormal = midNormal / std::sqrt(z); }
        V3 normTwistVec = ((midNormal * dt) * .5) * dot(midNormal, angVel1 + angVel2);
        const M3 prevTrsf = C->trsf;
        M3 midTrsf;
        V3 rt = normRotVec + normTwistVec;
        if (approxMask & 4) { midTrsf.setCol(0, prevNormal); midTrsf.setCol(1, prevTrsf.col(1)); }
        else { midTrsf.setCol(0, midNormal); midTrsf.setCol(1, prevTrsf.col(1) - cross(prevTrsf.col(1), rt) / 2.); }
        midTrsf.setCol(2, cross(midTrsf.col(0), midTrsf.col(1)));
        M3 currTrsf;
        currTrsf.setCol(0, currNormal);
        currTrsf.setCol(1, prevTrsf.col(1) - cross(midTrsf.col(1), rt));
        currTrsf.setCol(2, cross(currTrsf.col(0), currTrsf.col(1)));
        if (cfg.trsf_renorm > 0 && (step % cfg.trsf_renorm) == 0) {
            V3 c0 = currTrsf.col(0);
            { double z = sqn(c0); if (z > 0) c0 = c0 / std::sqrt(z); }
            V3 c1 = currTrsf.col(1);
            c1 = c1 - c0 * dot(c1, c0);
            { double z = sqn(c1); if (z > 0) c1 = c1 / std::sqrt(z); }
            currTrsf.setCol(0, c0); currTrsf.setCol(1, c1); currTrsf.setCol(2, cross(c0, c1));
        }
        V3 midContPt, midPos1, midPos2;
        if (approxMask & 8) { midContPt = contPt; midPos1 = pos1; midPos2 = pos2; }
        else { midContPt = .5 * (prevContPt + contPt); midPos1 = pos1 - (dt / 2.) * vel1; midPos2 = pos2 - (dt / 2.) * (vel2 + shiftVel2); }
        V3 c1x = (cfg.no_ratch && r1 > 0) ? r1 * midNormal : midContPt - midPos1;
        V3 c2x = (cfg.no_ratch && r2 > 0) ? (-r2) * midNormal : midContPt - midPos2;
        V3 relVel = ((vel2 + shiftVel2) + cross(angVel2, c2x)) - (vel1 + cross(angVel1, c1x));
        C->trsf = currTrsf;
        C->lvel = mulT(midTrsf, relVel);
        C->langVel = mulT(midTrsf, angVel2 - angVel1);
        C->uN = uN;
        C->cpos = contPt;
        C->cori = quatFromMat(C->trsf);
    }
    // Cg2_Sphere_Sphere_L6Geom::go, pkg/dem/Sphere.cpp:88-109
    bool cg2SS(Contact* C, const V3& shift2) {
        const Particle &s1 = par[C->pA], &s2 = par[C->pB];
        const double r1 = s1.radius, r2 = s2.radius;
        const Node &n1 = nodes[s1.nodes[0]], &n2 = nodes[s2.nodes[0]];
        V3 relPos = (n2.pos + shift2) - n1.pos;
        double dfr = std::abs(cfg.cg2_ss_dist_factor) * (r1 + r2);
        double unDistSq = sqn(relPos) - dfr * dfr;
        if (unDistSq > 0 && !C->isReal()) return false;
        double dist = std::sqrt(sqn(relPos));
        double uN = dist - (r1 + r2);
        V3 normal = relPos / dist;
        V3 contPt = n1.pos + (r1 + 0.5 * uN) * normal;
        handleSpheresLikeContact(C, n1.pos, n1.vel, n1.angVel, n2.pos + shift2, n2.vel, n2.angVel, normal, contPt, uN, r1, r2);
        return true;
    }
    // Cg2_Wall_Sphere_L6Geom::go, pkg/dem/Wall.cpp:45-79
    bool cg2WS(Contact* C, const V3& shift2) {
        if (cfg.periodic && cell.hasShear) throw std::logic_error("Cg2_Wall_Sphere_L6Geom does not handle periodic boundary conditions with skew (Scene.cell.trsf is not diagonal).");
        const Particle &w = par[C->pA], &s = par[C->pB];
        const double radius = s.radius; const int ax = w.axis, sense = w.sense;
        const Node &wn = nodes[w.nodes[0]], &sn = nodes[s.nodes[0]];
        V3 spherePos = sn.pos + shift2;
        double dist = spherePos[ax] - wn.pos[ax];
        if (!C->isReal() && std::abs(dist) > radius) return false;
        V3 contPt = spherePos; contPt[ax] = wn.pos[ax];
        V3 normal;
        if (sense == 0) {
            if (!C->geom) normal[ax] = dist > 0 ? 1. : -1.;
            else normal[ax] = C->trsf.m[ax][0];
        } else normal[ax] = (sense == 1 ? 1. : -1);
        double uN = normal[ax] * dist - radius;
        handleSpheresLikeContact(C, wn.pos, wn.vel, wn.angVel, spherePos, sn.vel, sn.angVel, normal, contPt, uN, -radius, radius);
        return true;
    }
    // CompUtils::closestSegmentPt, lib/base/CompUtils.cpp:57-63
    static V3 closestSegmentPt(const V3& P, const V3& A, const V3& B) {
        V3 BA = B - A;
        if (sqn(BA) == 0.) return A;
        double u = (dot(P, BA) - dot(A, BA)) / sqn(BA);
        return A + std::min(1., std::max(0., u)) * BA;
    }
    // CompUtils::triangleBarycentrics, lib/base/CompUtils.cpp:92-110 (2x2 normal equations, inverse via 1/det)
    static V3 triangleBarycentrics(const V3& x, const V3& A, const V3& B, const V3& C) {
        V3 vB = B - A, vC = C - A, vX = x - A;
        double m00 = dot(vB, vB), m01 = dot(vC, vB), m10 = dot(vB, vC), m11 = dot(vC, vC);
        double det = m00 * m11 - m10 * m01;
        double invdet = 1. / det;
        double i00 = m11 * invdet, i10 = -m10 * invdet, i01 = -m01 * invdet, i11 = m00 * invdet;
        double b0 = dot(vX, vB), b1 = dot(vX, vC);
        double u = i00 * b0 + i01 * b1, v = i10 * b0 + i11 * b1;
        return V3((1 - u) - v, u, v);
    }
    // Cg2_Facet_Sphere_L6Geom::go, pkg/dem/Facet.cpp:235-288 (+ Facet::getNormal :71-74, getOuterVectors :110-115,
    // interpolatePtLinAngVel :158-174)
    bool cg2FS(Contact* C, const V3& shift2) {
        const Particle &f = par[C->pA], &s = par[C->pB];
        const Node &sn = nodes[s.nodes[0]];
        const V3 sC = sn.pos + shift2;
        const V3 &p0 = nodes[f.nodes[0]].pos, &p1 = nodes[f.nodes[1]].pos, &p2 = nodes[f.nodes[2]].pos;
        V3 nn = cross(p1 - p0, p2 - p0);
        V3 fNormal = nn; { double z = sqn(nn); if (z > 0) fNormal = nn / std::sqrt(z); }
        double planeDist = dot(sC - p0, fNormal);
        if (std::abs(planeDist) > (s.radius + f.halfThick) && !C->isReal()) return false;
        V3 fC = sC - planeDist * fNormal;
        V3 outVec[3] = {cross(p1 - p0, nn), cross(p2 - p1, nn), cross(p0 - p2, nn)};
        const V3* pp[3] = {&p0, &p1, &p2};
        double ll[3];
        for (int i = 0; i < 3; i++) ll[i] = dot(outVec[i], fC - *pp[i]);
        int w = (ll[0] > 0 ? 1 : 0) + (ll[1] > 0 ? 2 : 0) + (ll[2] > 0 ? 4 : 0);
        V3 contPt;
        switch (w) {
            case 0: contPt = fC; break;
            case 1: contPt = closestSegmentPt(fC, p0, p1); break;
            case 2: contPt = closestSegmentPt(fC, p1, p2); break;
            case 4: contPt = closestSegmentPt(fC, p2, p0); break;
            case 3: contPt = p1; break;
            case 5: contPt = p0; break;
            case 6: contPt = p2; break;
            default: throw std::logic_error("Cg2_Facet_Sphere_L3Geom: Impossible sphere-facet intersection (all points are outside the edges). (please report bug)");
        }
        V3 normal = sC - contPt;
        double rh = s.radius + f.halfThick;
        if (sqn(normal) > rh * rh && !C->isReal()) return false;
        double dist = std::sqrt(sqn(normal));
        normal = normal / dist;
        if (f.halfThick > 0) contPt = contPt + normal * f.halfThick;
        double uN = (dist - s.radius) - f.halfThick;
        // interpolatePtLinAngVel(contPt)
        V3 a = triangleBarycentrics(contPt, p0, p1, p2);
        const V3 &v0 = nodes[f.nodes[0]].vel, &v1 = nodes[f.nodes[1]].vel, &v2 = nodes[f.nodes[2]].vel;
        V3 linVel = (a.x * v0 + a.y * v1) + a.z * v2;
        V3 angVel = (cross(p0 - contPt, v0) + cross(p1 - contPt, v1)) + cross(p2 - contPt, v2);
        if (!isZero(f.fakeVel)) {
            if (!std::isnan(f.fakeVel.x)) linVel = linVel + f.fakeVel;
            else linVel = dot(linVel, fNormal) * fNormal;
        }
        handleSpheresLikeContact(C, contPt, linVel, angVel, sC, sn.vel, sn.angVel, normal, contPt, uN, std::max(f.halfThick, s.radius), s.radius);
        return true;
    }

    // Cp2_FrictMat_FrictPhys::go/updateFrictPhys, pkg/dem/FrictMat.cpp:13-44
    void cp2Frict(Contact* C) {
        const Material &m1 = mats[par[C->pA].mat], &m2 = mats[par[C->pB].mat];
        double l0 = C->lens[0], l1 = C->lens[1], A = C->contA;
        C->phys = true;
        C->force = V3(); C->torque = V3();
        C->kn = 1 / (1 / (m1.young * A / l0) + 1 / (m2.young * A / l1));
        C->kt = .5 * (m1.ktDivKn + m2.ktDivKn) * C->kn;
        C->tanPhi = std::min(m1.tanPhi, m2.tanPhi);
    }
    // Cp2_FrictMat_HertzPhys::go, pkg/dem/Hertz.cpp:9-50
    void cp2Hertz(Contact* C) {
        const Material &m1 = mats[par[C->pA].mat], &m2 = mats[par[C->pB].mat];
        C->phys = true;
        C->force = V3(); C->torque = V3();
        const double r1 = C->lens[0], r2 = C->lens[1];
        const double E1 = m1.young, E2 = m2.young;
        const double nu1 = cfg.hz_poisson, nu2 = cfg.hz_poisson;
        C->K = (4 / 3.) * 1. / ((1 - nu1 * nu1) / E1 + (1 - nu2 * nu2) / E2);
        C->R = 1. / (1. / r1 + 1. / r2);
        double kn0 = C->K * std::sqrt(C->R);
        C->gamma = cfg.hz_gamma;
        C->alpha = cfg.hz_alpha;
        double G1 = E1 / (2 * (1 + nu1)), G2 = E2 / (2 * (1 + nu2));
        double G = .5 * (G1 + G2);
        double nu = .5 * (nu1 + nu2);
        C->kt0 = 2 * std::sqrt(4 * C->R) * G / (2 - nu);
        C->tanPhi = std::min(m1.tanPhi, m2.tanPhi);
        if (viscOn) {
            double ma = nodes[par[C->pA].nodes[0]].mass, mb = nodes[par[C->pB].nodes[0]].mass;
            double mbar = (ma <= 0 && mb > 0) ? mb : ((ma > 0 && mb <= 0) ? ma : (ma * mb) / (ma + mb));
            C->alpha_sqrtMK = std::max(0., viscAlphaConst * std::sqrt(mbar * kn0));
        } else C->alpha_sqrtMK = 0.0;
    }
    // Law2_L6Geom_FrictPhys_IdealElPl::go, pkg/dem/IdealElPl.cpp:12-122 (no energy tracking, no rolling)
    // (energy tracking: the "broken", "plast" and "elast" additions of :25-37, :58-72, :84-89)
    bool lawIdealElPl(Contact* C) {
        double uN = C->uN;
        if (uN > 0 && !cfg.no_break) {
            if (cfg.no_slip && cfg.track_energy) {
                const double Fn = C->kn * uN;
                const double fy = C->force.y + (cfg.dt * C->kt) * C->lvel.y, fz = C->force.z + (cfg.dt * C->kt) * C->lvel.z;
                C->en[2] = .5 * ((Fn * Fn) / C->kn + (fy * fy + fz * fz) / C->kt);
                C->enN[1] = 1;
            }
            return false;
        }
        C->torque = V3();
        C->force.x = C->kn * uN;
        if (cfg.no_frict || C->tanPhi == 0.) { C->force.y = 0; C->force.z = 0; }
        else {
            double vy = C->lvel.y, vz = C->lvel.z;
            C->force.y = C->force.y + (cfg.dt * C->kt) * vy;
            C->force.z = C->force.z + (cfg.dt * C->kt) * vz;
            double maxFt = std::abs(C->force.x) * C->tanPhi;
            if ((C->force.y * C->force.y + C->force.z * C->force.z) > maxFt * maxFt && !cfg.no_slip) {
                double FtNorm = std::sqrt(C->force.y * C->force.y + C->force.z * C->force.z);
                double ratio = maxFt / FtNorm;
                if (FtNorm == 0.) ratio = 0.;
                if (cfg.track_energy) C->en[1] = (C->kt != 0. ? (maxFt * (FtNorm - maxFt)) / C->kt : 0.);
                C->force.y = C->force.y * ratio; C->force.z = C->force.z * ratio;
            }
            if (std::isnan(std::max(std::max(C->force.x, C->force.y), C->force.z))) throw std::runtime_error("NaN force in contact (message above)?!");
        }
        if (cfg.track_energy) {
            double e = 0.5 * ((C->force.x * C->force.x) / C->kn +
                              (C->kt != 0. ? (C->force.y * C->force.y + C->force.z * C->force.z) / C->kt : 0.));
            if (std::isnan(e)) e = 0.;
            C->en[0] = e;
            C->enN[0] = 1;
        }
        return true;
    }
    // Law2_L6Geom_HertzPhys_DMT::go, pkg/dem/Hertz.cpp:58-182 (DMT branch alpha==0; Schwarz branch rejected)
    bool lawHertz(Contact* C) {
        const double dt = cfg.dt;
        const double velN = C->lvel.x, vy = C->lvel.y, vz = C->lvel.z;
        C->torque = V3();
        double kn0 = C->K * std::sqrt(C->R);
        C->kn = (3 / 2.) * kn0 * std::sqrt(-C->uN);
        double Fne, Fna = 0.;
        if (C->uN > 0) return false;
        double su = std::sqrt(-C->uN);
        Fne = -kn0 * (su * su * su);
        Fna = 4 * PI * C->R * C->gamma;
        double eta = (C->alpha_sqrtMK > 0 ? C->alpha_sqrtMK * std::sqrt(std::sqrt(std::max(-C->uN, 0.))) : 0.);
        double Fnv = eta * velN;
        if (cfg.hz_no_attraction && Fne + Fnv > 0) Fnv = -Fne;
        double Fn = (Fne + Fna) + Fnv;
        C->force.x = Fn;
        if (cfg.track_energy) C->en[3] = (Fnv * velN) * dt;  // viscN, :154
        C->kt = C->kt0 * std::sqrt(C->uN < 0 ? -C->uN : 0);
        double fy = (dt * C->kt) * vy, fz = (dt * C->kt) * vz;
        double maxFt = std::max(0., Fn) * C->tanPhi;
        if ((fy * fy + fz * fz) > maxFt * maxFt) {
            double FtNorm = std::sqrt(fy * fy + fz * fz);
            double ratio = maxFt / FtNorm;
            if (cfg.track_energy) C->en[1] = ((.5 * (FtNorm - maxFt) + maxFt) * (FtNorm - maxFt)) / C->kt;  // plast, :166
            fy = fy * ratio; fz = fz * ratio;
        } else {
            fy = fy + eta * vy; fz = fz + eta * vz;
            if (cfg.track_energy) C->en[4] = (eta * (vy * vy + vz * vz)) * dt;  // viscT, :171
        }
        C->force.y = fy; C->force.z = fz;
        if (cfg.track_energy && C->uN < 0) {
            // elast, :174-179: normalElasticEnergy(kn0,-uN) = kn0*(2/5)*pow(sqrt(-uN),5), with the
            // power written as a product
            C->en[0] = (kn0 * (2 / 5.)) * ((((su * su) * su) * su) * su) + (0.5 * (fy * fy + fz * fz)) / C->kt;
            C->enN[0] = 1;
        }
        return true;
    }
    // Contact::getForceTorqueBranch + ContactLoop::applyForceUninodal,
    // pkg/dem/Contact.cpp:24-34, pkg/dem/ContactLoop.cpp:261-267, DemData::addForceTorque pkg/dem/Particle.hpp:221
    void applyForceUninodal(const Contact* C, int pid, bool atomic) {
        const Particle& p = par[pid];
        if (p.nNodes() != 1) return;
        bool isPA = (C->pA == pid);
        double sign = isPA ? 1 : -1;
        V3 F = qrot(C->cori, C->force) * sign;
        V3 T = isZero(C->torque) ? V3() : qrot(C->cori, C->torque) * sign;
        Node& n = nodes[p.nodes[0]];
        V3 shift = (!isPA && cfg.periodic) ? cell.intrShiftPos(C->cellDist) : V3();
        V3 xc = C->cpos - (n.pos + shift);
        V3 tq = cross(xc, F) + T;
        if (atomic) {
#pragma omp atomic
            n.force.x += F.x;
#pragma omp atomic
            n.force.y += F.y;
#pragma omp atomic
            n.force.z += F.z;
#pragma omp atomic
            n.torque.x += tq.x;
#pragma omp atomic
            n.torque.y += tq.y;
#pragma omp atomic
            n.torque.z += tq.z;
        } else {
            n.force = n.force + F;
            n.torque = n.torque + tq;
        }
    }
    // ContactLoop::run, pkg/dem/ContactLoop.cpp:93-259
    void contactLoopRun() {
        for (auto& pl : pending) {  // ContactContainer::removeAllPending (no-op after the collider)
            for (Contact* c : pl) removeMaybe_fast(c);
            pl.clear();
        }
        stress = M3();
        const bool doStress = (cfg.eval_stress && cfg.periodic);
        const bool deterministic = cfg.deterministic;
        if (!deterministic && (step % 1000 == 0)) reorderContacts();
        long size = (long)linView.size();
        std::string ex;
#pragma omp parallel for schedule(guided) num_threads(nThreads)
        for (long i = 0; i < size; i++) {
            try {
                Contact* C = linView[i];
                for (int q = 0; q < 5; q++) C->en[q] = 0;
                C->enN[0] = C->enN[1] = 0;
                const bool fresh = (C->stepCreated == step);
                if (!C->isReal() && fresh) {
                    // functor order: DEFINE_FUNCTOR_ORDER_2D(Facet,Sphere) / (Wall,Sphere) put the non-sphere first
                    int tA = par[C->pA].shape, tB = par[C->pB].shape;
                    if (tA == SH_SPHERE && tB != SH_SPHERE) { std::swap(C->pA, C->pB); for (int k = 0; k < 3; k++) C->cellDist[k] *= -1; }
                    // Cg2_Sphere_Sphere_L6Geom::setMinDist00Sq pkg/dem/Sphere.cpp:83-85; others set -1
                    if (par[C->pA].shape == SH_SPHERE && par[C->pB].shape == SH_SPHERE) {
                        double d = std::abs(cfg.cg2_ss_dist_factor * (par[C->pA].radius + par[C->pB].radius));
                        C->minDist00Sq = d * d;
                    } else C->minDist00Sq = -1;
                }
                int tA = par[C->pA].shape, tB = par[C->pB].shape;
                V3 shift2 = cfg.periodic ? cell.intrShiftPos(C->cellDist) : V3();
                if (!C->isReal() && !fresh && C->minDist00Sq > 0 &&
                    sqn(nodes[par[C->pA].nodes[0]].pos - (nodes[par[C->pB].nodes[0]].pos + shift2)) > C->minDist00Sq) continue;
                bool geomCreated;
                if (tA == SH_SPHERE && tB == SH_SPHERE) geomCreated = cg2SS(C, shift2);
                else if (tA == SH_WALL && tB == SH_SPHERE) geomCreated = cg2WS(C, shift2);
                else if (tA == SH_FACET && tB == SH_SPHERE) geomCreated = cg2FS(C, shift2);
                else geomCreated = false;  // no functor for this shape pair
                if (!geomCreated) continue;
                if (!C->phys) C->stepCreated = (int)step;
                if (!C->phys) { if (cfg.phys == 0) cp2Frict(C); else cp2Hertz(C); }
                bool keep = (cfg.law == 0) ? lawIdealElPl(C) : lawHertz(C);
                if (!keep) { C->reset(); pending[tid()].push_back(C); }
                if (cfg.apply_forces && C->isReal() && !deterministic) {
                    applyForceUninodal(C, C->pA, true);
                    applyForceUninodal(C, C->pB, true);
                }
                if (doStress && C->isReal()) {
                    const V3 &pa = nodes[par[C->pA].nodes[0]].pos, &pb = nodes[par[C->pB].nodes[0]].pos;
                    V3 branch = pb - pa;
                    if (C->cellDist[0] != 0 || C->cellDist[1] != 0 || C->cellDist[2] != 0) branch = branch + cell.intrShiftPos(C->cellDist);
                    V3 F = qrot(C->cori, C->force);
#pragma omp critical
                    {
                        for (int a = 0; a < 3; a++) for (int b = 0; b < 3; b++) stress.m[a][b] += F[a] * branch[b];
                    }
                }
            } catch (std::exception& e) {
#pragma omp critical
                ex = e.what();
            }
        }
        if (!ex.empty()) throw std::runtime_error(ex);
        if (cfg.track_energy) {
            // EnergyTracker::add of every contact, summed in linView order; elast is reset every step
            double e[5] = {0, 0, 0, 0, 0};
            int n[2] = {0, 0};
            for (Contact* C : linView) {
                for (int q = 0; q < 5; q++) e[q] = e[q] + C->en[q];
                n[0] += C->enN[0]; n[1] += C->enN[1];
            }
            energy[EN_ELAST] = e[0];
            if (n[0]) ecreated[EN_ELAST] = 1;
            energy[EN_PLAST] += e[1];
            if (e[1] != 0) ecreated[EN_PLAST] = 1;
            energy[EN_BROKEN] += e[2];
            if (n[1]) ecreated[EN_BROKEN] = 1;
            energy[EN_VISCN] += e[3];
            if (e[3] != 0) ecreated[EN_VISCN] = 1;
            energy[EN_VISCT] += e[4];
            if (e[4] != 0) ecreated[EN_VISCT] = 1;
        }
        if (doStress) {
            stress = mdiv(stress, mdet(cell.hSize));
            // the work of the velocity gradient, ContactLoop.cpp:236-246
            const double vol = mdet(cell.hSize);
            if (cfg.track_energy) {
                const M3 midStress = mscale(madd(stress, prevStress), .5);
                const double midVol = !std::isnan(prevVol) ? .5 * (prevVol + vol) : vol;
                const M3 gm = mmul(cell.gradV, midStress);
                const double dW = ((-((gm.m[0][0] + gm.m[1][1]) + gm.m[2][2])) * cfg.dt) * midVol;
                energy[EN_GRADV] += dW;
                if (dW != 0) ecreated[EN_GRADV] = 1;
            }
            prevVol = vol;
            prevStress = stress;
        }
        if (deterministic && cfg.apply_forces) {
            for (Contact* C : linView) {
                if (!C->isReal()) continue;
                applyForceUninodal(C, C->pA, false);
                applyForceUninodal(C, C->pB, false);
            }
        }
    }
    // ContactLoop::reorderContacts, pkg/dem/ContactLoop.cpp:75-91
    void reorderContacts() {
        size_t N = linView.size();
        if (N < 2) return;
        size_t lowestReal = 0;
        for (size_t i = N - 1; i > lowestReal; i--) {
            if (!linView[i]->isReal()) continue;
            while (lowestReal < i && linView[lowestReal]->isReal()) lowestReal++;
            if (lowestReal == i) return;
            std::swap(linView[i], linView[lowestReal]);
            linView[i]->linIx = i; linView[lowestReal]->linIx = lowestReal;
        }
    }

    // ------------------------------------------------------------ Leapfrog
    // Leapfrog::run, pkg/dem/Leapfrog.cpp:103-255 (+ nonviscDamp2nd :32-34, computeAccel :36-47,
    // applyPeriodicCorrections :258-272, leapfrogTranslate :275-278, leapfrogSphericalRotate :280-288)
    void leapfrogRun() {
        const double dt = cfg.dt;
        const int homoDeform = cfg.periodic ? cell.homoDeform : -1;
        M3 dGradV = msub(cell.nextGradV, cell.gradV);
        M3 midGradV = mscale(madd(cell.gradV, cell.nextGradV), .5);
        M3 ImLL4hInv, IpLL4h, LmL; V3 deltaSpinVec;
        if (homoDeform == HOMO_GRADV2) {
            const M3 &pprevL = cell.gradV, &nnextL = cell.nextGradV;
            M3 q = mdiv(mscale(madd(nnextL, pprevL), dt), 4.);
            ImLL4hInv = minv(msub(M3::I(), q));
            IpLL4h = madd(M3::I(), q);
            LmL = msub(nnextL, pprevL);
            deltaSpinVec = -.5 * leviCivita(mscale(msub(pprevL, mtr(pprevL)), .5)) + .5 * leviCivita(mscale(msub(nnextL, mtr(nnextL)), .5));
        }
        const double damping = cfg.damping;
        const V3 g(cfg.gravity[0], cfg.gravity[1], cfg.gravity[2]);
        const bool hasGravity = !isZero(g);
        long n = (long)nodes.size();
        std::string ex;
        // Leapfrog.cpp:104: energies are tracked, except in the first step of a periodic scene
        // whose gradV is not the identity
        const bool track = cfg.track_energy && (!cfg.periodic || step > 0 || isIdentity(cell.gradV));
        // per node: kinetic (Etrans+Erot, or Etrans and Erot with kinSplit), grav, nonviscDamp, and
        // whether kinetic/grav were added
        std::vector<double> eK0, eK1, eGr, eDm;
        std::vector<char> eNk, eNg;
        if (track) { eK0.assign(n, 0); eK1.assign(n, 0); eGr.assign(n, 0); eDm.assign(n, 0); eNk.assign(n, 0); eNg.assign(n, 0); }
#pragma omp parallel for schedule(guided) num_threads(nThreads)
        for (long i = 0; i < n; i++) {
            Node& nd = nodes[i];
            if (nd.flags & CLUMP_CLUMPED) continue;
            bool damp = (damping != 0. && !(nd.flags & DAMPING_SKIP));
            V3& f = nd.force; V3& t = nd.torque;
            const bool blockedAll = (nd.flags & DOF_ALL) == DOF_ALL;
            V3 pvfE = nd.vel, pvaE = nd.angVel;
            if (track) {
                // Leapfrog::doDampingDissipation, :52-63 (velocities of the previous half step)
                if (damp && !(nd.flags & ENERGY_SKIP)) {
                    const double a = (std::abs(nd.vel.x) * std::abs(f.x) + std::abs(nd.vel.y) * std::abs(f.y)) + std::abs(nd.vel.z) * std::abs(f.z);
                    const double b = (std::abs(nd.angVel.x) * std::abs(t.x) + std::abs(nd.angVel.y) * std::abs(t.y)) + std::abs(nd.angVel.z) * std::abs(t.z);
                    eDm[i] = ((a * damping) * dt) + ((b * damping) * dt);
                }
                // Leapfrog::doGravityWork, :66-73
                if (hasGravity && !(nd.flags & GRAVITY_SKIP)) {
                    double gr = 0;
                    if ((nd.flags & DOF_ALL) == 0) gr = ((-dot(g, nd.vel)) * nd.mass) * dt;
                    else for (int k = 0; k < 3; k++) if (!(nd.flags & (1u << k))) gr = gr - ((g[k] * nd.vel[k]) * nd.mass) * dt;
                    eGr[i] = gr; eNg[i] = 1;
                }
                // the fluctuation velocities Leapfrog computes for free nodes; for fully blocked
                // nodes the reference reads vectors it never set, here the same expressions stand in
                if (cfg.periodic) { pvfE = cell.pprevFluctVel(nd.pos, nd.vel, dt); pvaE = cell.pprevFluctAngVel(nd.angVel); }
            }
            const bool aspherical = !(nd.inertia.x == nd.inertia.y && nd.inertia.y == nd.inertia.z);
            const bool useAspherical = aspherical && ((nd.flags & DOF_RXRYRZ) != DOF_RXRYRZ);
            if (useAspherical) {
#pragma omp critical
                ex = "aspherical integration is not part of the restated path";
                continue;
            }
            V3 linAccel, angAccel;
            if (!blockedAll) {
                if ((nd.flags & DOF_ALL) == 0) linAccel = f / nd.mass;
                else for (int k = 0; k < 3; k++) if (!(nd.flags & (1u << k))) linAccel[k] = 0. + f[k] / nd.mass;
                V3 pvf, pva;
                if (cfg.periodic) { pvf = cell.pprevFluctVel(nd.pos, nd.vel, dt); pva = cell.pprevFluctAngVel(nd.angVel); }
                else { pvf = nd.vel; pva = nd.angVel; }
                if (damp) for (int k = 0; k < 3; k++) {
                    double s = f[k] * (pvf[k] + (0.5 * dt) * linAccel[k]);
                    double sg = s < 0 ? -1 : (s > 0 ? 1 : 0);
                    linAccel[k] = linAccel[k] * (1 - damping * sg);
                }
                if (homoDeform == HOMO_GRADV2) nd.vel = mul(ImLL4hInv, (mul(LmL, nd.pos) + mul(IpLL4h, nd.vel)) + linAccel * dt);
                else nd.vel = nd.vel + dt * linAccel;
                if (!isZero(nd.inertia)) {
                    if ((nd.flags & DOF_ALL) == 0) angAccel = V3(t.x / nd.inertia.x, t.y / nd.inertia.y, t.z / nd.inertia.z);
                    else for (int k = 0; k < 3; k++) if (!(nd.flags & (1u << (k + 3)))) angAccel[k] = 0. + t[k] / nd.inertia[k];
                    if (damp) for (int k = 0; k < 3; k++) {
                        double s = t[k] * (pva[k] + (0.5 * dt) * angAccel[k]);
                        double sg = s < 0 ? -1 : (s > 0 ? 1 : 0);
                        angAccel[k] = angAccel[k] * (1 - damping * sg);
                    }
                    nd.angVel = nd.angVel + dt * angAccel;
                    if (homoDeform == HOMO_GRADV2) nd.angVel = nd.angVel - deltaSpinVec;
                }
            } else {
                if (homoDeform == HOMO_GRADV2) nd.vel = mul(ImLL4hInv, mul(LmL, nd.pos) + mul(IpLL4h, nd.vel));
            }
            if (homoDeform >= 0 && homoDeform != HOMO_GRADV2) {
                if (homoDeform == HOMO_VEL || homoDeform == HOMO_VEL_2ND) {
                    if (homoDeform == HOMO_VEL_2ND) nd.vel = nd.vel + mul(midGradV, nd.vel - (dt / 2.) * linAccel) * dt;
                    nd.vel = nd.vel + mul(dGradV, nd.pos);
                } else if (homoDeform == HOMO_POS) nd.pos = nd.pos + mul(cell.nextGradV, nd.pos) * dt;
            }
            if (track && !(nd.flags & ENERGY_SKIP)) {
                // Leapfrog::doKineticEnergy, :75-97 (spherical nodes), on-step velocities
                const V3 cv = pvfE + (.5 * dt) * linAccel, cw = pvaE + (.5 * dt) * angAccel;
                const double et = (.5 * nd.mass) * sqn(cv);
                double er = 0.5 * ((cw.x * (nd.inertia.x * cw.x) + cw.y * (nd.inertia.y * cw.y)) + cw.z * (nd.inertia.z * cw.z));
                if (std::isnan(er) || std::isinf(std::max(std::max(nd.inertia.x, nd.inertia.y), nd.inertia.z))) er = 0;
                if (cfg.kin_split) { eK0[i] = et; eK1[i] = er; }
                else eK0[i] = et + er;
                eNk[i] = 1;
            }
            nd.pos = nd.pos + nd.vel * dt;
            V3 axis = nd.angVel;
            if (!isZero(axis)) {
                double angle = std::sqrt(sqn(axis));
                axis = axis / angle;
                double ha = 0.5 * (angle * dt);
                double s = std::sin(ha);
                Q q{std::cos(ha), s * axis.x, s * axis.y, s * axis.z};
                nd.ori = qmul(q, nd.ori);
            }
            qnormalize(nd.ori);
            if (cfg.reset) {
                nd.force = (hasGravity && !(nd.flags & GRAVITY_SKIP)) ? nd.mass * g : V3();
                nd.torque = V3();
            }
        }
        if (!ex.empty()) throw std::runtime_error(ex);
        if (cfg.track_energy) {
            // EnergyTracker::add of every node, summed in node order; kinetic is reset every step
            double k0 = 0, k1 = 0, gr = 0, dm = 0; int nk = 0, ng = 0;
            if (track)
                for (long i = 0; i < n; i++) { k0 = k0 + eK0[i]; k1 = k1 + eK1[i]; gr = gr + eGr[i]; dm = dm + eDm[i]; nk += eNk[i]; ng += eNg[i]; }
            if (cfg.kin_split) {
                energy[EN_KINTRANS] = k0; energy[EN_KINROT] = k1;
                if (nk) ecreated[EN_KINTRANS] = ecreated[EN_KINROT] = 1;
            } else {
                energy[EN_KINETIC] = k0;
                if (nk) ecreated[EN_KINETIC] = 1;
            }
            energy[EN_GRAV] += gr;
            if (ng) ecreated[EN_GRAV] = 1;
            energy[EN_DAMP] += dm;
            if (dm != 0) ecreated[EN_DAMP] = 1;
        }
    }

    // ------------------------------------------------------------ DynDt
    // PeriodicEngine counters (core/Engine.hpp:136-151), Scene.nextDt and the simulation time
    // since the scene's time 0 (PeriodicEngine's virtual clock)
    long ddNDone = 0, ddStepLast = -1, ddStepPrev = -1, ddNEvals = 0;
    double ddVirtLast = 0, ddVirtPrev = 0;
    double ddDt = std::numeric_limits<double>::quiet_NaN(), ddCritDt = Inf;
    double nextDt = std::numeric_limits<double>::quiet_NaN(), timeAbs = 0;
    // PeriodicEngine::isActivated, core/Engine.cpp:169-194 (realPeriod, the wall clock, is not restated)
    bool dynDtActivated() {
        const double virtNow = timeAbs;
        const long stepNow = step;
        const bool initNow = ddStepLast < 0;
        if (initNow) { ddVirtLast = virtNow; ddStepLast = stepNow; }
        const bool due = (cfg.dyndt_virt_period > 0 && virtNow - ddVirtLast >= cfg.dyndt_virt_period) ||
                         (cfg.dyndt_step_period > 0 && ((stepNow - ddStepLast >= cfg.dyndt_step_period) ||
                                                        (cfg.dyndt_step_modulo && stepNow % cfg.dyndt_step_period == 0)));
        if ((cfg.dyndt_n_do < 0 || ddNDone < cfg.dyndt_n_do) && due) {
            ddVirtPrev = ddVirtLast; ddVirtLast = virtNow;
            ddStepPrev = ddStepLast; ddStepLast = stepNow;
            if (initNow && !cfg.dyndt_init_run) return false;
            ddNDone++;
            return true;
        }
        return false;
    }
    // DynDt::critDt_stiffness with nodalCritDtSq and nodalStiffAdd, pkg/dem/DynDt.cpp:17-76: for
    // every node, the stiffness of the real contacts of each particle of the node (Particle.contacts,
    // ordered by the id of the other particle), then 2*min(m/|ktrans_i|, I_i/|krot_i|) over the free
    // axes; the square root of the minimum over nodes. pow(x,2) of the reference is restated as x*x.
    double dynDtCritStiffness() {
        std::vector<std::vector<std::pair<int, Contact*>>> byPar(par.size());
        for (Contact* C : linView) {
            if (!C->isReal()) continue;
            byPar[C->pA].push_back({C->pB, C});
            byPar[C->pB].push_back({C->pA, C});
        }
        for (auto& v : byPar)
            std::sort(v.begin(), v.end(), [](const std::pair<int, Contact*>& a, const std::pair<int, Contact*>& b) { return a.first < b.first; });
        std::vector<std::vector<int>> parRef(nodes.size());
        for (size_t p = 0; p < par.size(); p++)
            for (int k = 0; k < par[p].nNodes(); k++) parRef[par[p].nodes[k]].push_back((int)p);
        double ret = Inf;
        for (size_t i = 0; i < nodes.size(); i++) {
            const Node& nd = nodes[i];
            double r = Inf;
            if ((nd.flags & DOF_ALL) != DOF_ALL) {
                V3 kt, kr;
                for (int p : parRef[i]) {
                    for (const auto& e : byPar[p]) {
                        const Contact* C = e.second;
                        const int ix = (C->pA == p) ? 0 : 1;
                        const V3 n = qrot(C->cori, V3(1, 0, 0));
                        const V3 n2(n.x * n.x, n.y * n.y, n.z * n.z);
                        kt = kt + V3(n2.x * (C->kn - C->kt) + C->kt, n2.y * (C->kn - C->kt) + C->kt, n2.z * (C->kn - C->kt) + C->kt);
                        const double sc = (C->lens[ix] * C->lens[ix]) * C->kt;
                        kr = kr + V3(sc * (n2.y + n2.z), sc * (n2.z + n2.x), sc * (n2.x + n2.y));
                    }
                }
                for (int a = 0; a < 3; a++)
                    if (kt[a] != 0 && nd.mass > 0. && !(nd.flags & (1u << a))) r = std::min(r, nd.mass / std::abs(kt[a]));
                for (int a = 0; a < 3; a++)
                    if (kr[a] != 0 && nd.inertia[a] > 0. && !(nd.flags & (8u << a))) r = std::min(r, nd.inertia[a] / std::abs(kr[a]));
                r = 2 * r;
            }
            ret = std::min(ret, r);
        }
        return std::sqrt(ret);
    }
    // DynDt::run, pkg/dem/DynDt.cpp:93-113
    void dynDtRun() {
        const double crDt = dynDtCritStiffness();
        ddCritDt = crDt;
        ddNEvals++;
        if (std::isinf(crDt)) return;
        const int nSteps = (int)(step - ddStepPrev);
        const double maxNewDt = cfg.dt * std::pow(1. + cfg.dyndt_max_rel_inc, nSteps);
        const double ndt = std::min(crDt * cfg.dt_safety, maxNewDt);
        if (!cfg.dyndt_dry_run) {
            if (ndt != cfg.dt) { ddDt = std::numeric_limits<double>::quiet_NaN(); nextDt = ndt; }
        } else ddDt = ndt;
    }

    // Scene::doOneStep, core/Scene.cpp:319-389 with the engine list Leapfrog, InsertionSortCollider,
    // ContactLoop and, if configured, DynDt
    void doOneStep() {
        if (cfg.periodic) cell.integrateAndUpdate(cfg.dt);
        leapfrogRun();
        colliderRun();
        contactLoopRun();
        if (cfg.dyndt && dynDtActivated()) dynDtRun();
        if (cfg.periodic) cell.setNextGradV();
        step++;
        time += cfg.dt;
        timeAbs += cfg.dt;
        if (!std::isnan(nextDt)) { cfg.dt = nextDt; nextDt = std::numeric_limits<double>::quiet_NaN(); }
    }
    void prepare() {
        size_t T = (size_t)nThreads;
        makeLater.resize(T); makeLaterPeri.resize(T); removeLater.resize(T); pending.resize(T);
        sqrt5 = std::sqrt(5.);
        viscOn = (cfg.hz_en > 0 && cfg.hz_en < 1.);
        if (viscOn) { double le = std::log(cfg.hz_en); viscAlphaConst = -sqrt5 * le / (std::sqrt(le * le + PI * PI)); }
        else viscAlphaConst = 0;
    }
};

}  // namespace wo

using namespace wo;

extern "C" {
void* wo_create(void) {
    Scene* s = new Scene();
    std::memset(&s->cfg, 0, sizeof(s->cfg));
    s->cfg.trsf_renorm = 100; s->cfg.apply_forces = 1; s->cfg.cg2_ss_dist_factor = 1; s->cfg.bo1_sphere_dist_factor = -1;
#ifdef _OPENMP
    s->nThreads = 1;
#endif
    return s;
}
void wo_destroy(void* s) { delete (Scene*)s; }
const char* wo_last_error(void* s) { return ((Scene*)s)->err.c_str(); }
int wo_set_threads(void* s, int n) { ((Scene*)s)->nThreads = n < 1 ? 1 : n; return 0; }
int wo_set_config(void* sp, const wo_config* c) {
    Scene* s = (Scene*)sp;
    s->cfg = *c;
    s->step = c->step;
    s->ddNDone = c->dyndt_n_done; s->ddStepLast = c->dyndt_step_last; s->ddStepPrev = c->dyndt_step_prev;
    s->ddVirtLast = c->dyndt_virt_last; s->ddVirtPrev = c->dyndt_virt_prev;
    s->nextDt = (c->next_dt > 0 && std::isfinite(c->next_dt)) ? c->next_dt : std::numeric_limits<double>::quiet_NaN();
    s->timeAbs = c->time;
    if (c->law == 1 && c->hz_alpha != 0) { s->err = "Law2_L6Geom_HertzPhys_DMT: the Schwarz branch (alpha!=0) is not part of the restated path"; return -4; }
    if (c->periodic) {
        Cell& cl = s->cell;
        for (int i = 0; i < 9; i++) {
            cl.hSize.m[i / 3][i % 3] = c->cell_hsize[i]; cl.trsf.m[i / 3][i % 3] = c->cell_trsf[i];
            cl.gradV.m[i / 3][i % 3] = c->cell_gradv[i]; cl.nextGradV.m[i / 3][i % 3] = c->cell_next_gradv[i];
        }
        cl.homoDeform = c->homo_deform;
        cl.pprevHsize = cl.hSize;
        cl.W = mscale(msub(cl.gradV, mtr(cl.gradV)), .5);
        cl.spinVec = .5 * leviCivita(cl.W);
        try { cl.integrateAndUpdate(0); } catch (std::exception& e) { s->err = e.what(); return -1; }
    }
    return 0;
}
int wo_set_materials(void* sp, int32_t n, const double* density, const double* young, const double* tan_phi, const double* kt_div_kn) {
    Scene* s = (Scene*)sp;
    s->mats.resize(n);
    for (int i = 0; i < n; i++) s->mats[i] = Material{density[i], young[i], tan_phi[i], kt_div_kn[i]};
    return 0;
}
int wo_set_nodes(void* sp, int64_t n, const double* pos, const double* ori, const double* vel, const double* ang_vel,
                 const double* force, const double* torque, const double* mass, const double* inertia, const uint32_t* flags) {
    Scene* s = (Scene*)sp;
    s->nodes.resize(n);
    for (int64_t i = 0; i < n; i++) {
        Node& d = s->nodes[i];
        d.pos = V3(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]);
        d.ori = Q{ori[4 * i], ori[4 * i + 1], ori[4 * i + 2], ori[4 * i + 3]};
        d.vel = V3(vel[3 * i], vel[3 * i + 1], vel[3 * i + 2]);
        d.angVel = V3(ang_vel[3 * i], ang_vel[3 * i + 1], ang_vel[3 * i + 2]);
        d.force = V3(force[3 * i], force[3 * i + 1], force[3 * i + 2]);
        d.torque = V3(torque[3 * i], torque[3 * i + 1], torque[3 * i + 2]);
        d.mass = mass[i];
        d.inertia = V3(inertia[3 * i], inertia[3 * i + 1], inertia[3 * i + 2]);
        d.flags = flags[i];
    }
    return 0;
}
int wo_set_particles(void* sp, int64_t n, const int32_t* shape, const int32_t* nodes3, const double* radius, const int32_t* wall_axis,
                     const int32_t* wall_sense, const double* half_thick, const double* fake_vel, const int32_t* mat, const uint32_t* mask) {
    Scene* s = (Scene*)sp;
    s->par.resize(n);
    for (int64_t i = 0; i < n; i++) {
        Particle& p = s->par[i];
        p.shape = shape[i];
        for (int k = 0; k < 3; k++) p.nodes[k] = nodes3[3 * i + k];
        p.radius = radius[i]; p.axis = wall_axis[i]; p.sense = wall_sense[i]; p.halfThick = half_thick[i];
        p.fakeVel = V3(fake_vel[3 * i], fake_vel[3 * i + 1], fake_vel[3 * i + 2]);
        p.mat = mat[i]; p.mask = mask[i]; p.hasBound = false; p.maxD2 = 0;
    }
    return 0;
}
int wo_run(void* sp, int64_t n_steps) {
    Scene* s = (Scene*)sp;
    try {
        s->prepare();
        for (int64_t i = 0; i < n_steps; i++) s->doOneStep();
    } catch (std::exception& e) { s->err = e.what(); return -1; }
    return 0;
}
int wo_collide_only(void* sp) {
    Scene* s = (Scene*)sp;
    try { s->prepare(); s->colliderRun(true); } catch (std::exception& e) { s->err = e.what(); return -1; }
    return 0;
}
int wo_get_nodes(void* sp, double* pos, double* ori, double* vel, double* ang_vel, double* force, double* torque) {
    Scene* s = (Scene*)sp;
    for (size_t i = 0; i < s->nodes.size(); i++) {
        const Node& d = s->nodes[i];
        if (pos) { pos[3 * i] = d.pos.x; pos[3 * i + 1] = d.pos.y; pos[3 * i + 2] = d.pos.z; }
        if (ori) { ori[4 * i] = d.ori.w; ori[4 * i + 1] = d.ori.x; ori[4 * i + 2] = d.ori.y; ori[4 * i + 3] = d.ori.z; }
        if (vel) { vel[3 * i] = d.vel.x; vel[3 * i + 1] = d.vel.y; vel[3 * i + 2] = d.vel.z; }
        if (ang_vel) { ang_vel[3 * i] = d.angVel.x; ang_vel[3 * i + 1] = d.angVel.y; ang_vel[3 * i + 2] = d.angVel.z; }
        if (force) { force[3 * i] = d.force.x; force[3 * i + 1] = d.force.y; force[3 * i + 2] = d.force.z; }
        if (torque) { torque[3 * i] = d.torque.x; torque[3 * i + 1] = d.torque.y; torque[3 * i + 2] = d.torque.z; }
    }
    return 0;
}
int wo_get_stats(void* sp, wo_stats* o) {
    Scene* s = (Scene*)sp;
    o->step = s->step; o->n_full_runs = s->nFullRuns; o->n_contacts = (int64_t)s->linView.size();
    int64_t r = 0; for (auto* c : s->linView) r += c->isReal();
    o->n_real = r; o->time = s->time; o->verlet_dist = s->verletDist;
    for (int i = 0; i < 9; i++) o->stress[i] = s->stress.m[i / 3][i % 3];
    return 0;
}
int wo_get_energy(void* sp, double* values, int32_t* created) {
    Scene* s = (Scene*)sp;
    for (int k = 0; k < EN_N; k++) { values[k] = s->energy[k]; created[k] = s->ecreated[k]; }
    return 0;
}
int wo_get_dyndt(void* sp, wo_dyndt_state* o) {
    Scene* s = (Scene*)sp;
    o->dt = s->cfg.dt; o->next_dt = s->nextDt; o->dyndt_dt = s->ddDt; o->crit_dt = s->ddCritDt;
    o->n_done = s->ddNDone; o->step_last = s->ddStepLast; o->step_prev = s->ddStepPrev; o->n_evals = s->ddNEvals;
    o->virt_last = s->ddVirtLast; o->virt_prev = s->ddVirtPrev;
    return 0;
}
int wo_get_cell(void* sp, double* hsize, double* trsf, double* gradv) {
    Scene* s = (Scene*)sp;
    for (int i = 0; i < 9; i++) {
        if (hsize) hsize[i] = s->cell.hSize.m[i / 3][i % 3];
        if (trsf) trsf[i] = s->cell.trsf.m[i / 3][i % 3];
        if (gradv) gradv[i] = s->cell.gradV.m[i / 3][i % 3];
    }
    return 0;
}
int64_t wo_num_contacts(void* s) { return (int64_t)((Scene*)s)->linView.size(); }
int wo_get_contacts(void* sp, int32_t* id_lo, int32_t* id_hi, int32_t* id_a, int32_t* real, int32_t* cell_dist, double* fglob,
                    double* local, double* cpt, double* trsf) {
    Scene* s = (Scene*)sp;
    std::vector<Contact*> cc = s->linView;
    std::sort(cc.begin(), cc.end(), [](const Contact* a, const Contact* b) { return ckey(a->pA, a->pB) < ckey(b->pA, b->pB); });
    for (size_t i = 0; i < cc.size(); i++) {
        const Contact* C = cc[i];
        id_lo[i] = std::min(C->pA, C->pB); id_hi[i] = std::max(C->pA, C->pB); id_a[i] = C->pA; real[i] = C->isReal();
        // cellDist is reported for the (lo,hi) orientation
        int sg = (C->pA == id_lo[i]) ? 1 : -1;
        for (int k = 0; k < 3; k++) cell_dist[3 * i + k] = sg * C->cellDist[k];
        const bool r = C->isReal();
        V3 F = r ? qrot(C->cori, C->force) : V3();
        V3 L = r ? C->force : V3();
        V3 P = r ? C->cpos : V3();
        fglob[3 * i] = F.x; fglob[3 * i + 1] = F.y; fglob[3 * i + 2] = F.z;
        local[3 * i] = L.x; local[3 * i + 1] = L.y; local[3 * i + 2] = L.z;
        cpt[3 * i] = P.x; cpt[3 * i + 1] = P.y; cpt[3 * i + 2] = P.z;
        for (int k = 0; k < 9; k++) trsf[9 * i + k] = r ? C->trsf.m[k / 3][k % 3] : 0.;
    }
    return 0;
}
int wo_get_aabbs(void* sp, double* mn, double* mx) {
    Scene* s = (Scene*)sp;
    for (size_t i = 0; i < s->par.size(); i++)
        for (int k = 0; k < 3; k++) { mn[3 * i + k] = s->par[i].mn[k]; mx[3 * i + k] = s->par[i].mx[k]; }
    return 0;
}
int wo_kinetic_energy(void* sp, double* ek) {
    Scene* s = (Scene*)sp;
    double e = 0;
    for (auto& n : s->nodes) {
        if ((n.flags & DOF_ALL) == DOF_ALL) continue;
        e += .5 * n.mass * sqn(n.vel) + .5 * dot(n.angVel, V3(n.inertia.x * n.angVel.x, n.inertia.y * n.angVel.y, n.inertia.z * n.angVel.z));
    }
    *ek = e;
    return 0;
}
}
