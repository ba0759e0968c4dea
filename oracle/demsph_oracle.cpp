// FP64 host oracle of the coupled DEM-SPH step.
//
// TEST INFRASTRUCTURE - the oracle, never the product.  Only tests/,
// __graft_entry__.smoke() and bench.py's CPU-baseline leg load this library.
//
// A CPU restatement, in FP64 and in plain loops (OpenMP over particles), of
// the reference's step as its kernels compute it: the same hashed grid, the
// same half pair lists in the same order with reverse spans, the same spring
// history remap, the same force expressions and the same step schedule.
// Every function cites the reference code it restates.  Two deliberate
// departures, both because the reference's behaviour is not defined:
//   * continuity (core/integrate.cu:55-161) updates dRho in place while
//     neighbours read it; here every particle reads the values as of the pass
//     start (what the GPU does when the whole grid is resident at once);
//   * findStartAndEnd (core/neighborSearch.cu:56-69) races on the last cell's
//     end; here it takes the non-racing value n.
// Pinned against the reference itself compiled for the CPU (oracle/_ref,
// tests/golden/): integer artefacts identical, floating point to ~1e-12.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../include/demsph_gb300.h"

namespace {

struct V3 {
    double x, y, z;
};
inline V3 mk(double x, double y, double z) { return V3{x, y, z}; }
inline V3 operator+(V3 a, V3 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
inline V3 operator-(V3 a, V3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
inline V3 operator-(V3 a) { return mk(-a.x, -a.y, -a.z); }
inline V3 operator*(V3 a, double s) { return mk(a.x * s, a.y * s, a.z * s); }
inline V3 operator*(double s, V3 a) { return mk(a.x * s, a.y * s, a.z * s); }
inline V3 operator/(V3 a, double s) { return mk(a.x / s, a.y / s, a.z / s); }
inline V3& operator+=(V3& a, V3 b) { a.x += b.x; a.y += b.y; a.z += b.z; return a; }
inline V3& operator-=(V3& a, V3 b) { a.x -= b.x; a.y -= b.y; a.z -= b.z; return a; }
inline V3& operator*=(V3& a, double s) { a.x *= s; a.y *= s; a.z *= s; return a; }
inline double dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V3 cross(V3 a, V3 b) { return mk(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
inline double len(V3 v) { return std::sqrt(dot(v, v)); }
inline V3 unit(V3 v) { return len(v) > 0 ? v / std::sqrt(dot(v, v)) : v; }
const double PI = 3.1415926535897931;

// Rodrigues rotation of v by the rotation vector w (core/myVec.h:98-109).
inline V3 rotate(V3 v, V3 w)
{
    const double a = len(w);
    if (a < 1.e-10) return v;
    const V3 k = w / a;
    return v * std::cos(a) + cross(k, v) * std::sin(a) + k * (dot(k, v) * (1 - std::cos(a)));
}

struct Quat {
    double q0, q1, q2, q3;
};
struct Sym {
    double xx, yy, zz, xy, xz, yz;
};
inline V3 mul(const Sym& m, V3 v)
{
    return mk(m.xx * v.x + m.xy * v.y + m.xz * v.z, m.xy * v.x + m.yy * v.y + m.yz * v.z,
              m.xz * v.x + m.yz * v.y + m.zz * v.z);
}
// R(q) invI R(q)^T written out as in core/myMat.h:102-127.
Sym rotateInverseInertia(const Quat& q, const Sym& I)
{
    const double q0 = q.q0, q1 = q.q1, q2 = q.q2, q3 = q.q3;
    const double a = 1 - 2 * q2 * q2 - 2 * q3 * q3, b = 2 * q1 * q2 - 2 * q0 * q3, c = 2 * q1 * q3 + 2 * q0 * q2;
    const double d = 2 * q1 * q2 + 2 * q0 * q3, e = 1 - 2 * q1 * q1 - 2 * q3 * q3, f = 2 * q2 * q3 - 2 * q0 * q1;
    const double g = 2 * q1 * q3 - 2 * q0 * q2, h = 2 * q2 * q3 + 2 * q0 * q1, i = 1 - 2 * q1 * q1 - 2 * q2 * q2;
    Sym m;
    m.xx = I.xx * a * a + 2 * I.xy * a * b + 2 * I.xz * a * c + I.yy * b * b + 2 * I.yz * b * c + I.zz * c * c;
    m.xy = d * (I.xx * a + I.xy * b + I.xz * c) + e * (I.xy * a + I.yy * b + I.yz * c) +
           f * (I.xz * a + I.yz * b + I.zz * c);
    m.xz = g * (I.xx * a + I.xy * b + I.xz * c) + h * (I.xy * a + I.yy * b + I.yz * c) +
           i * (I.xz * a + I.yz * b + I.zz * c);
    m.yy = I.xx * d * d + 2 * I.xy * d * e + 2 * I.xz * d * f + I.yy * e * e + 2 * I.yz * e * f + I.zz * f * f;
    m.yz = g * (I.xx * d + I.xy * e + I.xz * f) + h * (I.xy * d + I.yy * e + I.yz * f) +
           i * (I.xz * d + I.yz * e + I.zz * f);
    m.zz = I.xx * g * g + 2 * I.xy * g * h + 2 * I.xz * g * i + I.yy * h * h + 2 * I.yz * h * i + I.zz * i * i;
    return m;
}
// First-order quaternion update (core/myQua.h:45-54).
Quat quatRotate(const Quat& q, V3 w, double dt)
{
    const V3 v = w * dt;
    Quat n{q.q0 + 0.5 * (-q.q1 * v.x - q.q2 * v.y - q.q3 * v.z), q.q1 + 0.5 * (q.q0 * v.x + q.q3 * v.y - q.q2 * v.z),
           q.q2 + 0.5 * (-q.q3 * v.x + q.q0 * v.y + q.q1 * v.z), q.q3 + 0.5 * (q.q2 * v.x - q.q1 * v.y + q.q0 * v.z)};
    const double l = std::sqrt(n.q0 * n.q0 + n.q1 * n.q1 + n.q2 * n.q2 + n.q3 * n.q3);
    if (l > 0) { n.q0 /= l; n.q1 /= l; n.q2 /= l; n.q3 /= l; }
    return n;
}

// ---- SPH kernel and contact laws (core/SPHKernelDEMContactModel.h) ----

// Wendland C2, 3-D, support 2h (SPHKernelDEMContactModel.h:5-13).
inline double wendland(double r, double h)
{
    const double q = r / h;
    if (q >= 2.0) return 0.0;
    const double sigma = 21.0 / (16.0 * PI * h * h * h);
    const double t = 1.0 - 0.5 * q;
    return sigma * std::pow(t, 4) * (1.0 + 2.0 * q);
}
// Its gradient (SPHKernelDEMContactModel.h:15-32).
inline V3 gradWendland(V3 rij, double h)
{
    const double r = len(rij);
    if (r < 1.e-10 || r >= 2.0 * h) return mk(0, 0, 0);
    const double q = r / h;
    const double sigma = 21.0 / (16.0 * PI * h * h * h);
    const double t = 1.0 - 0.5 * q;
    const double dWdq = (-2.0 * std::pow(t, 3) * (1.0 + 2.0 * q) + 2.0 * std::pow(t, 4));
    const double dWdr = sigma * dWdq / h;
    return (dWdr / r) * rij;
}

// Incremental parallel bond (SPHKernelDEMContactModel.h:115-168); returns 1 if intact.
int parallelBond(double& Fn, double& Tt, V3& Fs, V3& Tb, V3 nPrev, V3 n, V3 vc, V3 wA, V3 wB, double rA, double rB,
                 double dt, double gamma, double E, double knks, double sigma, double C, double mu)
{
    const V3 th1 = cross(nPrev, n);
    Fs = rotate(Fs, th1);
    Tb = rotate(Tb, th1);
    const V3 th2 = dot(0.5 * (wA + wB) * dt, n) * n;
    Fs = rotate(Fs, th2);
    Tb = rotate(Tb, th2);
    const double rmin = rA < rB ? rA : rB;
    const double br = gamma * rmin;
    const double A = br * br * PI;
    const double I = br * br * br * br / 4. * PI;
    const double J = 2 * I;
    const double kn = E / (rA + rB);
    const double ks = kn / knks;
    V3 dn = dot(vc, n) * n * dt;
    V3 dtg = vc * dt - dn;
    Fn -= dot(dn * kn * A, n);
    Fs -= dtg * ks * A;
    const V3 wr = wA - wB;
    dn = dot(wr, n) * n * dt;
    dtg = wr * dt - dn;
    Tt -= dot(dn * ks * J, n);
    Tb -= dtg * kn * I;
    const double sN = -Fn / A + len(Tb) / I * br;
    const double sS = len(Fs) / A + std::fabs(Tt) / J * br;
    int bonded = 1;
    if (sigma > 0 && sN > sigma) bonded = 0;
    else if (C > 0 && sS > C - mu * sN) bonded = 0;
    return bonded;
}

// Tangential spring with Coulomb cap (SPHKernelDEMContactModel.h:170-193).
V3 slideRollSpring(V3 prev, V3 vel, V3 n, V3 Fn, double mu, double k, double c, double dt)
{
    V3 s = mk(0, 0, 0);
    if (mu > 0) {
        V3 p1 = prev - dot(prev, n) * n;
        const double a = len(p1);
        if (a > 1.e-10) p1 *= len(prev) / a;
        s = p1 + vel * dt;
        V3 F = -k * s - c * vel;
        const double aF = len(F), aN = len(Fn);
        if (aF > mu * aN) {
            F *= mu * aN / aF;
            s = -(F + c * vel) / k;
        }
    }
    return s;
}
// Torsion spring (SPHKernelDEMContactModel.h:195-212).
V3 torsionSpring(V3 prev, V3 vel, V3 n, V3 Fn, double mu, double k, double c, double dt)
{
    V3 s = mk(0, 0, 0);
    if (mu > 0) {
        s = dot(prev + vel * dt, n) * n;
        V3 F = -k * s - c * vel;
        const double aF = len(F), aN = len(Fn);
        if (aF > mu * aN) {
            F *= mu * aN / aF;
            s = -(F + c * vel) / k;
        }
    }
    return s;
}

// Shared tail of the linear and Hertz-Mindlin laws (SPHKernelDEMContactModel.h:241-260, 299-318).
void springForces(V3& F, V3& T, V3& es, V3& er, V3& et, V3 vc, V3 wr, V3 n, double delta, double R, double dt,
                  double kn, double ks, double kr, double kt, double cn, double cs, double cr, double ct,
                  double mus, double mur, double mut)
{
    const V3 vn = dot(vc, n) * n;
    const V3 Fn = kn * delta * n - vn * cn;
    const V3 vs = vc - vn;
    es = slideRollSpring(es, vs, n, Fn, mus, ks, cs, dt);
    const V3 Fs = -ks * es - cs * vs;
    const V3 vr = -R * cross(n, wr);
    er = slideRollSpring(er, vr, n, Fn, mur, kr, cr, dt);
    const V3 Fr = -kr * er - cr * vr;
    const V3 Tr = R * cross(n, Fr);
    const double D = 2 * R;
    const V3 vt = D * dot(wr, n) * n;
    et = torsionSpring(et, vt, n, Fn, mut, kt, ct, dt);
    const V3 Ft = -kt * et - ct * vt;
    const V3 Tt = D * Ft;
    F = Fn + Fs;
    T = Tr + Tt;
}

struct Tables {
    int nMat = 0;
    std::vector<double> hz, ln, bd;  // 8, 11, 6 per slot
    int slot(int a, int b) const
    {
        if (a >= nMat || b >= nMat) return -1;
        int i = a, j = b;
        if (a > b) { i = b; j = a; }
        return (i * (2 * nMat - i + 1)) / 2 + j - i;
    }
};

// Contact-law dispatch used by pair and wall contacts (core/integrate.cu:463-505).
void contactLaw(const Tables& t, int c, V3& F, V3& T, V3& es, V3& er, V3& et, V3 vc, V3 wr, V3 n, double delta,
                double m, double R, double dt)
{
    const double* L = &t.ln[11 * c];
    if (L[0] > 1.e-10) {  // LinearContact (SPHKernelDEMContactModel.h:214-268)
        if (delta > 0) {
            const double cn = 2. * L[4] * std::sqrt(m * L[0]), cs = 2. * L[5] * std::sqrt(m * L[1]);
            const double cr = 2. * L[6] * std::sqrt(m * L[2]), ct = 2. * L[7] * std::sqrt(m * L[3]);
            springForces(F, T, es, er, et, vc, wr, n, delta, R, dt, L[0], L[1], L[2], L[3], cn, cs, cr, ct, L[8],
                         L[9], L[10]);
        } else {
            es = er = et = mk(0, 0, 0);
        }
    } else {  // HertzianMindlinContact (SPHKernelDEMContactModel.h:270-326)
        const double* H = &t.hz[8 * c];
        const double logR = std::log(H[2]);
        const double D = -logR / std::sqrt(logR * logR + PI * PI);
        if (delta > 0) {
            const double kn = 4. / 3. * H[0] * std::sqrt(R * delta);
            const double ks = 8. * H[1] * std::sqrt(R * delta);
            const double cn = 2. * std::sqrt(5. / 6.) * D * std::sqrt(m * kn);
            const double cs = 2. * std::sqrt(5. / 6.) * D * std::sqrt(m * ks);
            const double kr = ks * H[3], kt = ks * H[4];
            const double cr = 2. * std::sqrt(5. / 6.) * D * std::sqrt(m * kr);
            const double ct = 2. * std::sqrt(5. / 6.) * D * std::sqrt(m * kt);
            springForces(F, T, es, er, et, vc, wr, n, delta, R, dt, kn, ks, kr, kt, cn, cs, cr, ct, H[5], H[6], H[7]);
        } else {
            es = er = et = mk(0, 0, 0);
        }
    }
}

struct Grid {
    V3 minB, maxB, cs;
    int gx = 1, gy = 1, gz = 1, num = 1;
    inline void cellOf(V3 p, int& x, int& y, int& z) const
    {
        x = int((p.x - minB.x) / cs.x);
        y = int((p.y - minB.y) / cs.y);
        z = int((p.z - minB.z) / cs.z);
    }
    inline int key(V3 p) const  // calculatePointHash (core/neighborSearch.cu:19-36)
    {
        if (minB.x <= p.x && p.x < maxB.x && minB.y <= p.y && p.y < maxB.y && minB.z <= p.z && p.z < maxB.z) {
            int x, y, z;
            cellOf(p, x, y, z);
            return z * gy * gx + y * gx + x;
        }
        return num - 1;
    }
};

// Cell spans after a stable sort by key (buildHashSpans, core/neighborSearch.cu:71-87).
struct Spans {
    std::vector<int> value, index, start, end;
    void build(const std::vector<int>& keys, int nCells)
    {
        const int n = (int)keys.size();
        index.resize(n);
        std::iota(index.begin(), index.end(), 0);
        std::stable_sort(index.begin(), index.end(), [&](int a, int b) { return keys[a] < keys[b]; });
        value.resize(n);
        for (int k = 0; k < n; ++k) value[k] = keys[index[k]];
        start.assign(nCells, -1);
        end.assign(nCells, -1);
        for (int k = 0; k < n; ++k) {
            if (k == 0 || value[k] != value[k - 1]) {
                start[value[k]] = k;
                if (k > 0) end[value[k - 1]] = k;
            }
        }
        if (n > 0) end[value[n - 1]] = n;
    }
};

struct PairList {
    std::vector<int> prefix;                // inclusive, per pointed object
    std::vector<int> pointed, pointing;
    Spans rev;                              // pairs sorted by pointing object
    int num() const { return (int)pointed.size(); }
};

struct Oracle {
    int fixes = 0;
    Grid grid;
    double domOrg[3] = {0, 0, 0}, domSize[3] = {0, 0, 0};  // setSpatialGrids' domain (re-gridding on append)
    V3 g;
    Tables tab;
    // fluid
    int nf = 0;
    std::vector<V3> fpos, fvel, facc;
    std::vector<double> fh, rho0, drho, cs, nu, sumW0;
    // solid
    int ns = 0;
    std::vector<V3> spos, svel, sacc, snorm, storq, sw;
    std::vector<double> seff, srad, sinvm;
    std::vector<int> smat, sclu, sclump, sdum;
    // clump
    int nc = 0;
    std::vector<V3> cpos, cvel, cacc, cw, ctorq;
    std::vector<Quat> cq;
    std::vector<Sym> cinvI;
    std::vector<double> cinvm;
    std::vector<int> cstart, cend;
    // walls
    int nw = 0;
    std::vector<V3> wp, wn;
    std::vector<int> wmat;
    std::vector<V3> wslide, wroll, wtors;  // ns * nw
    // neighbour structures
    Spans fcell, scell;
    PairList ff, fs, ss;
    std::vector<V3> fsForce;
    std::vector<V3> ssF, ssT, ssS, ssR, ssTo;
    // bonds
    std::vector<int> bA, bB, bOn;
    std::vector<double> bFn, bTt;
    std::vector<V3> bFs, bTb, bN, bP;
    std::string err;
};

V3 at3(const double* p, int i) { return p ? mk(p[3 * i], p[3 * i + 1], p[3 * i + 2]) : mk(0, 0, 0); }

// dataBase::setSpatialGrids (core/dataBase.cpp:415-432).
void setGrid(Oracle& o, const demsph_scene& s)
{
    double mf = 0, ms = 0;
    for (int i = 0; i < o.nf; ++i) mf = std::max(mf, o.fh[i]);
    for (int i = 0; i < o.ns; ++i) ms = std::max(ms, o.seff[i]);
    const double cell = 2 * std::max(mf, ms);
    const V3 org = mk(s.domain_origin[0], s.domain_origin[1], s.domain_origin[2]);
    const V3 size = mk(s.domain_size[0], s.domain_size[1], s.domain_size[2]);
    Grid& G = o.grid;
    G.minB = org;
    G.maxB = org + size;
    G.gx = size.x > cell ? int(size.x / cell) : 1;
    G.gy = size.y > cell ? int(size.y / cell) : 1;
    G.gz = size.z > cell ? int(size.z / cell) : 1;
    G.cs = mk(size.x / double(G.gx), size.y / double(G.gy), size.z / double(G.gz));
    G.num = G.gx * G.gy * G.gz + 1;
}

// ---- neighbour search (core/neighborSearch.cu) ----

void hashAll(Oracle& o)  // updateGridCellStartEnd (:89-113)
{
    std::vector<int> kf(o.nf), ks(o.ns);
#pragma omp parallel for
    for (int i = 0; i < o.nf; ++i) kf[i] = o.grid.key(o.fpos[i]);
#pragma omp parallel for
    for (int i = 0; i < o.ns; ++i) ks[i] = o.grid.key(o.spos[i]);
    o.fcell.build(kf, o.grid.num);
    o.scell.build(ks, o.grid.num);
}

// Walks the 27 stencil cells of a point the way the reference does
// (neighborSearch.cu:135-149): cell coordinates by truncation, linear hash,
// hashes outside [0, num) skipped.
template <class F>
void forStencil(const Grid& G, V3 p, F&& f)
{
    int x, y, z;
    G.cellOf(p, x, y, z);
    for (int zz = -1; zz <= 1; ++zz)
        for (int yy = -1; yy <= 1; ++yy)
            for (int xx = -1; xx <= 1; ++xx) {
                const int h = (z + zz) * G.gy * G.gx + (y + yy) * G.gx + (x + xx);
                if (h < 0 || h >= G.num) continue;
                f(h);
            }
}

// Two-pass CSR build: visit(A, emit) calls emit(B) for every pair (A, B) in order.
template <class Visit>
void buildCSR(int n, PairList& L, Visit&& visit)
{
    std::vector<int> cnt(n, 0);
#pragma omp parallel for schedule(dynamic, 256)
    for (int a = 0; a < n; ++a) {
        int c = 0;
        visit(a, [&](int) { ++c; });
        cnt[a] = c;
    }
    L.prefix.resize(n);
    int run = 0;
    for (int a = 0; a < n; ++a) {
        run += cnt[a];
        L.prefix[a] = run;
    }
    L.pointed.assign(run, -1);
    L.pointing.assign(run, -1);
#pragma omp parallel for schedule(dynamic, 256)
    for (int a = 0; a < n; ++a) {
        int w = a ? L.prefix[a - 1] : 0;
        visit(a, [&](int b) {
            L.pointed[w] = a;
            L.pointing[w] = b;
            ++w;
        });
    }
}

// Fluid lists: setFluidInteractionsKernel (neighborSearch.cu:115-220).
void buildFluidLists(Oracle& o)
{
    const Grid& G = o.grid;
    buildCSR(o.nf, o.ff, [&](int a, auto&& emit) {
        const V3 pa = o.fpos[a];
        const double ra = o.fh[a];
        forStencil(G, pa, [&](int h) {
            const int st = o.fcell.start[h];
            if (st == -1) return;
            for (int k = st; k < o.fcell.end[h]; ++k) {
                const int b = o.fcell.index[k];
                if (a >= b) continue;
                const double r = std::fmax(ra, o.fh[b]);
                if (2 * r - len(pa - o.fpos[b]) >= 0.) emit(b);
            }
        });
    });
    buildCSR(o.nf, o.fs, [&](int a, auto&& emit) {
        const V3 pa = o.fpos[a];
        const double ra = o.fh[a];
        forStencil(G, pa, [&](int h) {
            const int st = o.scell.start[h];
            if (st == -1) return;
            for (int k = st; k < o.scell.end[h]; ++k) {
                const int b = o.scell.index[k];
                if (2 * ra - len(pa - o.spos[b]) >= 0.) emit(b);
            }
        });
    });
    // reverse spans: pairs sorted by the object pointed to (neighborSearch.cu:345-354)
    o.ff.rev.build(o.ff.pointing, o.nf);
    o.fs.rev.build(o.fs.pointing, o.ns);
    o.fsForce.assign(o.fs.num(), mk(0, 0, 0));
}

// Solid list with spring history: setSolid2SolidInteractionsKernel
// (neighborSearch.cu:222-312), history from the previous list (save(),
// core/deviceStructs.h:693-706).
void buildSolidList(Oracle& o)
{
    const PairList prev = o.ss;
    const std::vector<V3> pS = o.ssS, pR = o.ssR, pT = o.ssTo;
    const Grid& G = o.grid;
    buildCSR(o.ns, o.ss, [&](int a, auto&& emit) {
        if (o.sdum[a] == 1) return;
        const V3 pa = o.spos[a];
        const double ra = o.seff[a];
        forStencil(G, pa, [&](int h) {
            const int st = o.scell.start[h];
            if (st == -1) return;
            for (int k = st; k < o.scell.end[h]; ++k) {
                const int b = o.scell.index[k];
                if (o.sdum[b] == 1) continue;
                if (a >= b) continue;
                if (o.sclump[a] >= 0 && o.sclump[a] == o.sclump[b]) continue;
                if (o.sinvm[a] < 1.e-10 && o.sinvm[b] < 1.e-10) continue;
                if (o.seff[b] + ra - len(pa - o.spos[b]) >= 0.) emit(b);
            }
        });
    });
    const int np = o.ss.num();
    o.ssF.assign(np, mk(0, 0, 0));
    o.ssT.assign(np, mk(0, 0, 0));
    o.ssS.assign(np, mk(0, 0, 0));
    o.ssR.assign(np, mk(0, 0, 0));
    o.ssTo.assign(np, mk(0, 0, 0));
#pragma omp parallel for
    for (int k = 0; k < np; ++k) {
        const int a = o.ss.pointed[k], b = o.ss.pointing[k];
        if (prev.rev.start.empty() || b >= (int)prev.rev.start.size()) continue;
        const int st = prev.rev.start[b];
        if (st == -1) continue;
        for (int j = st; j < prev.rev.end[b]; ++j) {
            const int j1 = prev.rev.index[j];
            if (prev.pointed[j1] == a) {
                o.ssS[k] = pS[j1];
                o.ssR[k] = pR[j1];
                o.ssTo[k] = pT[j1];
                break;
            }
        }
    }
    o.ss.rev.build(o.ss.pointing, o.ns);
}

// neighborSearch (neighborSearch.cu:314-382).
void neighborSearch(Oracle& o, int iStep, int gap)
{
    hashAll(o);
    if (iStep % gap == 0 && o.nf > 0) buildFluidLists(o);
    if (o.ns > 0) buildSolidList(o);
}

// ---- fluid (core/integrate.cu:3-421) ----

// Shepard sum of fluid i over its lists (integrate.cu:3-43).
double shepardSum(const Oracle& o, int i)
{
    const V3 ri = o.fpos[i];
    const double hi = o.fh[i];
    const double V0i = std::pow(hi / 1.3, 3);
    double sumW = wendland(0, hi);
    for (int k = i ? o.ff.prefix[i - 1] : 0; k < o.ff.prefix[i]; ++k)
        sumW += wendland(len(ri - o.fpos[o.ff.pointing[k]]), hi);
    if (o.ff.rev.start[i] != -1)
        for (int k = o.ff.rev.start[i]; k < o.ff.rev.end[i]; ++k)
            sumW += wendland(len(ri - o.fpos[o.ff.pointed[o.ff.rev.index[k]]]), hi);
    for (int k = i ? o.fs.prefix[i - 1] : 0; k < o.fs.prefix[i]; ++k) {
        const int a = o.fs.pointing[k];
        const double V0a = std::pow(2. * o.srad[a], 3);
        sumW += wendland(len(ri - o.spos[a]), hi) * V0a / V0i;
    }
    return sumW;
}

// Shepard density re-initialisation (integrate.cu:3-53).
void densityReinit(Oracle& o, int iStep)
{
#pragma omp parallel for
    for (int i = 0; i < o.nf; ++i) {
        const double sumW = shepardSum(o, i);
        const double rhoStar = o.rho0[i] + o.drho[i];
        if (iStep == 1) {
            o.sumW0[i] = sumW;
        } else {
            const double rho1 = std::fmax(rhoStar, o.rho0[i] * sumW / o.sumW0[i]);
            o.drho[i] = rho1 - o.rho0[i];
        }
    }
}

// Fluid partner term of the Riemann continuity equation (integrate.cu:75-103).
inline double continuityFluidTerm(const Oracle& o, const std::vector<double>& dr, int i, int j, V3 ri, V3 vi, double hi,
                                  double rhoi, double ci, double Pi)
{
    const V3 rj = o.fpos[j], vj = o.fvel[j];
    const double hj = o.fh[j], rho0j = o.rho0[j], dRhoj = dr[j], rhoj = rho0j + dRhoj, cj = o.cs[j];
    const double Pj = dRhoj * cj * cj;
    const double mj = std::pow(hj / 1.3, 3) * o.rho0[j];
    const double Vj = mj / rhoj;
    const V3 rij = ri - rj;
    const double h = 0.5 * (hi + hj), c = 0.5 * (ci + cj);
    const V3 e = unit(rij);
    const V3 dW = gradWendland(rij, h);
    const double UL = dot(vi, -e), UR = dot(vj, -e);
    const double Ustar = (rhoi * UL + rhoj * UR + (Pi - Pj) / c) / (rhoi + rhoj);
    const V3 vstar = (Ustar - (rhoi * UL + rhoj * UR) / (rhoi + rhoj)) * (-e) + (rhoi * vi + rhoj * vj) / (rhoi + rhoj);
    return 2 * rhoi * Vj * dot(vi - vstar, dW);
}

// Riemann continuity + density integration (integrate.cu:55-161), reading
// the pass-start densities for every partner.
void continuity(Oracle& o, double dt)
{
    const std::vector<double> dr = o.drho;
#pragma omp parallel for
    for (int i = 0; i < o.nf; ++i) {
        const V3 ri = o.fpos[i], vi = o.fvel[i];
        const double hi = o.fh[i], rho0i = o.rho0[i], dRhoi = dr[i], rhoi = rho0i + dRhoi, ci = o.cs[i];
        const double Pi = dRhoi * ci * ci;
        double dd = 0.;
        for (int k = i ? o.ff.prefix[i - 1] : 0; k < o.ff.prefix[i]; ++k)
            dd += continuityFluidTerm(o, dr, i, o.ff.pointing[k], ri, vi, hi, rhoi, ci, Pi);
        if (o.ff.rev.start[i] != -1)
            for (int k = o.ff.rev.start[i]; k < o.ff.rev.end[i]; ++k)
                dd += continuityFluidTerm(o, dr, i, o.ff.pointed[o.ff.rev.index[k]], ri, vi, hi, rhoi, ci, Pi);
        for (int k = i ? o.fs.prefix[i - 1] : 0; k < o.fs.prefix[i]; ++k) {
            const int a = o.fs.pointing[k];
            const V3 ra = o.spos[a], va = o.svel[a];
            const double Va = std::pow(2. * o.srad[a], 3);
            const double ha = 2.6 * o.srad[a];
            const double h = 0.5 * (hi + ha), c = ci;
            const V3 ria = ri - ra;
            const V3 e = unit(ri - ra);
            const V3 dW = gradWendland(ria, h);
            const V3 aa = o.sacc[a], na = o.snorm[a];
            const double Pa = Pi + rhoi * std::fmax(0., dot(o.g - aa, na)) * dot(ria, na);
            const double rhoa = Pa / (c * c) + rho0i;
            const V3 vstar = (Pi - Pa) / c / (rhoi + rhoa) * (-e) + (rhoi * vi + rhoa * (2 * va - vi)) / (rhoi + rhoa);
            dd += 2 * rhoi * Va * dot(vi - vstar, dW);
        }
        o.drho[i] = dr[i] + dt * dd;
    }
}

// Fluid partner term of the Riemann momentum equation (integrate.cu:185-213).
inline V3 momentumFluidTerm(const Oracle& o, int j, V3 ri, V3 vi, double hi, double rhoi, double ci, double Pi,
                            double gi, double mi, double Vi)
{
    const V3 rj = o.fpos[j], vj = o.fvel[j];
    const double hj = o.fh[j], rho0j = o.rho0[j], dRhoj = o.drho[j], rhoj = rho0j + dRhoj, cj = o.cs[j];
    const double Pj = dRhoj * cj * cj;
    const double gj = o.nu[j] * rhoj;
    const double mj = std::pow(hj / 1.3, 3) * o.rho0[j];
    const double Vj = mj / rhoj;
    const V3 rij = ri - rj;
    const double h = 0.5 * (hi + hj), c = 0.5 * (ci + cj);
    const V3 dW = gradWendland(rij, h);
    const V3 e = unit(rij);
    const double UL = dot(vi, -e), UR = dot(vj, -e);
    const double beta = std::fmin(3. * std::fmax(UL - UR, 0.), c);
    const double Ps = (rhoi * Pj + rhoj * Pi + rhoi * rhoj * beta * (UL - UR)) / (rhoi + rhoj);
    return -2 / mi * Vi * Vj * Ps * dW + 2 / mi * Vi * Vj * 2 * gi * gj / (gi + gj) * (vi - vj) / len(rij) * dot(e, dW);
}

// Solid partner term shared by momentum and the coupling force
// (integrate.cu:251-277 and 282-329); returns the acceleration contribution.
inline V3 solidPartnerTerm(const Oracle& o, int a, V3 ri, V3 vi, double hi, double rhoi, double ci, double Pi,
                           double rho0i, double gi, double mi, double Vi)
{
    const V3 ra = o.spos[a], va = o.svel[a];
    const double Va = std::pow(2. * o.srad[a], 3);
    const double ha = 2.6 * o.srad[a];
    const double h = 0.5 * (hi + ha), c = ci;
    const V3 ria = ri - ra;
    const V3 e = unit(ria);
    const V3 dW = gradWendland(ria, h);
    const V3 aa = o.sacc[a], na = o.snorm[a];
    const double UL = dot(vi, -na), UR = dot((2 * va - vi), -na);
    const double Pa = Pi + rhoi * std::fmax(0., dot(o.g - aa, na)) * dot(ria, na);
    const double rhoa = Pa / (c * c) + rho0i;
    const double beta = std::fmin(3. * std::fmax(UL - UR, 0.), c);
    const double Ps = (rhoi * Pa + rhoa * Pi + rhoi * rhoa * beta * (UL - UR)) / (rhoi + rhoa);
    return -2 / mi * Vi * Va * Ps * dW + 2 / mi * Vi * Va * gi * (vi - (2 * va - vi)) / len(ria) * dot(e, dW);
}

void momentum(Oracle& o)  // integrate.cu:163-280
{
#pragma omp parallel for
    for (int i = 0; i < o.nf; ++i) {
        const V3 ri = o.fpos[i], vi = o.fvel[i];
        const double hi = o.fh[i], rho0i = o.rho0[i], dRhoi = o.drho[i], rhoi = rho0i + dRhoi, ci = o.cs[i];
        const double Pi = dRhoi * ci * ci;
        const double gi = o.nu[i] * rhoi;
        const double mi = std::pow(hi / 1.3, 3) * rho0i;
        const double Vi = mi / rhoi;
        V3 dv = mk(0, 0, 0);
        for (int k = i ? o.ff.prefix[i - 1] : 0; k < o.ff.prefix[i]; ++k)
            dv += momentumFluidTerm(o, o.ff.pointing[k], ri, vi, hi, rhoi, ci, Pi, gi, mi, Vi);
        if (o.ff.rev.start[i] != -1)
            for (int k = o.ff.rev.start[i]; k < o.ff.rev.end[i]; ++k)
                dv += momentumFluidTerm(o, o.ff.pointed[o.ff.rev.index[k]], ri, vi, hi, rhoi, ci, Pi, gi, mi, Vi);
        for (int k = i ? o.fs.prefix[i - 1] : 0; k < o.fs.prefix[i]; ++k)
            dv += solidPartnerTerm(o, o.fs.pointing[k], ri, vi, hi, rhoi, ci, Pi, rho0i, gi, mi, Vi);
        o.facc[i] = dv + o.g;
    }
}

void fluid2SolidForce(Oracle& o)  // calFluid2SolidForce (integrate.cu:282-330)
{
    const int np = o.fs.num();
#pragma omp parallel for
    for (int k = 0; k < np; ++k) {
        const int i = o.fs.pointed[k];
        const V3 ri = o.fpos[i], vi = o.fvel[i];
        const double hi = o.fh[i], rho0i = o.rho0[i], dRhoi = o.drho[i], rhoi = rho0i + dRhoi, ci = o.cs[i];
        const double Pi = dRhoi * ci * ci;
        const double gi = o.nu[i] * rhoi;
        const double mi = std::pow(hi / 1.3, 3) * rho0i;
        const double Vi = mi / rhoi;
        V3 f = mk(0, 0, 0);
        f += solidPartnerTerm(o, o.fs.pointing[k], ri, vi, hi, rhoi, ci, Pi, rho0i, gi, mi, Vi);
        o.fsForce[k] = f * mi;
    }
}

void fluidKick(Oracle& o, double dt)
{
#pragma omp parallel for
    for (int i = 0; i < o.nf; ++i) o.fvel[i] += dt * o.facc[i];
}
void fluidDrift(Oracle& o, double dt)
{
#pragma omp parallel for
    for (int i = 0; i < o.nf; ++i) o.fpos[i] += dt * o.fvel[i];
}

// fluidIntegrate (integrate.cu:385-421).
void fluidIntegrate(Oracle& o, double dt, int iStep, int gap)
{
    const double dtf = dt * double(gap);
    if (o.nf > 0 && (iStep % (5 * gap) == 0 || iStep == 1)) densityReinit(o, iStep);
    if (iStep % gap == 0 && o.nf > 0) {
        continuity(o, 0.5 * dtf);
        fluidDrift(o, 0.5 * dtf);
    }
    fluid2SolidForce(o);
    if (iStep % gap == 0 && o.nf > 0) {
        momentum(o);
        fluidKick(o, dtf);
        fluidDrift(o, 0.5 * dtf);
        continuity(o, 0.5 * dtf);
    }
}

// ---- solids (core/integrate.cu:423-998) ----

// Contact geometry of pair (i, j) (integrate.cu:434-442, 758-765, 820-825).
inline void pairGeometry(const Oracle& o, int i, int j, V3& n, double& delta, V3& rc)
{
    const double ri = o.srad[i], rj = o.srad[j];
    const V3 pi = o.spos[i], pj = o.spos[j];
    n = unit(pi - pj);
    delta = ri + rj - len(pi - pj);
    rc = pj + (rj - 0.5 * delta) * n;
}

void pairContacts(Oracle& o, double dt)  // calSolidContactForceTorque (integrate.cu:423-512)
{
    const int np = o.ss.num();
#pragma omp parallel for
    for (int k = 0; k < np; ++k) {
        const int i = o.ss.pointed[k], j = o.ss.pointing[k];
        const double ri = o.srad[i], rj = o.srad[j];
        V3 n, rc;
        double delta;
        pairGeometry(o, i, j, n, delta, rc);
        const double R = ri * rj / (ri + rj);
        const double m = 1. / (o.sinvm[i] + o.sinvm[j]);
        const V3 pi = o.spos[i], pj = o.spos[j];
        const V3 vc = o.svel[i] + cross(o.sw[i], rc - pi) - (o.svel[j] + cross(o.sw[j], rc - pj));
        const V3 wr = o.sw[i] - o.sw[j];
        V3 F = mk(0, 0, 0), T = mk(0, 0, 0);
        V3 es = o.ssS[k], er = o.ssR[k], et = o.ssTo[k];
        const int c = o.tab.slot(o.smat[i], o.smat[j]);
        contactLaw(o.tab, c, F, T, es, er, et, vc, wr, n, delta, m, R, dt);
        o.ssF[k] = F;
        o.ssT[k] = T;
        o.ssS[k] = es;
        o.ssR[k] = er;
        o.ssTo[k] = et;
    }
}

void bondContacts(Oracle& o, double dt)  // calSolidBondedForceTorque (integrate.cu:717-804)
{
    const int nb = (int)o.bA.size();
    // Two bonds never share a pair (one bond per pair, created from the pair
    // list), so the pair updates below do not collide.
#pragma omp parallel for
    for (int b = 0; b < nb; ++b) {
        if (o.bOn[b] == 0) {
            o.bFn[b] = 0;
            o.bTt[b] = 0;
            o.bFs[b] = mk(0, 0, 0);
            o.bTb[b] = mk(0, 0, 0);
            o.bN[b] = mk(0, 0, 0);
            continue;
        }
        const int i = o.bA[b], j = o.bB[b];
        int kk = -1;
        for (int k = i ? o.ss.prefix[i - 1] : 0; k < o.ss.prefix[i]; ++k)
            if (o.ss.pointing[k] == j) {
                kk = k;
                break;
            }
        if (kk < 0) {
            o.bOn[b] = 0;
            continue;
        }
        const double ri = o.srad[i], rj = o.srad[j];
        V3 n, rc;
        double delta;
        pairGeometry(o, i, j, n, delta, rc);
        const V3 n0 = o.bN[b];
        const V3 pi = o.spos[i], pj = o.spos[j];
        const V3 vc = o.svel[i] + cross(o.sw[i], rc - pi) - (o.svel[j] + cross(o.sw[j], rc - pj));
        const int c = o.tab.slot(o.smat[i], o.smat[j]);
        const double* B = &o.tab.bd[6 * c];
        double Fn = o.bFn[b], Tt = o.bTt[b];
        V3 Fs = o.bFs[b], Tb = o.bTb[b];
        o.bOn[b] = parallelBond(Fn, Tt, Fs, Tb, n0, n, vc, o.sw[i], o.sw[j], ri, rj, dt, B[0], B[1], B[2], B[3], B[4],
                                B[5]);
        o.bFn[b] = Fn;
        o.bFs[b] = Fs;
        o.bTt[b] = Tt;
        o.bTb[b] = Tb;
        o.bN[b] = n;
        o.bP[b] = rc;
        o.ssF[kk] += Fn * n + Fs;
        o.ssT[kk] += Tt * n + Tb;
    }
}

void solidForceGather(Oracle& o)  // calSolidForceTorque (integrate.cu:806-858)
{
#pragma omp parallel for
    for (int i = 0; i < o.ns; ++i) {
        const V3 pi = o.spos[i];
        V3 F = mk(0, 0, 0), T = mk(0, 0, 0);
        for (int k = i ? o.ss.prefix[i - 1] : 0; k < o.ss.prefix[i]; ++k) {
            const int j = o.ss.pointing[k];
            V3 n, rc;
            double delta;
            pairGeometry(o, i, j, n, delta, rc);
            F += o.ssF[k];
            T += o.ssT[k] + cross(rc - pi, o.ssF[k]);
        }
        if (o.ss.rev.start[i] != -1)
            for (int k = o.ss.rev.start[i]; k < o.ss.rev.end[i]; ++k) {
                const int k1 = o.ss.rev.index[k];
                const int j = o.ss.pointed[k1];
                // the reference evaluates this pair's geometry from i's side
                const double rI = o.srad[i], rJ = o.srad[j];
                const V3 pj = o.spos[j];
                const V3 n = unit(pi - pj);
                const double delta = rI + rJ - len(pi - pj);
                const V3 rc = pj + (rJ - 0.5 * delta) * n;
                F -= o.ssF[k1];
                T -= o.ssT[k1];
                T -= cross(rc - pi, o.ssF[k1]);
            }
        if (!o.fs.rev.start.empty() && o.fs.rev.start[i] != -1)
            for (int k = o.fs.rev.start[i]; k < o.fs.rev.end[i]; ++k) F -= o.fsForce[o.fs.rev.index[k]];
        o.sacc[i] = F * o.sinvm[i] + o.g * double(o.sinvm[i] > 0. && o.sclump[i] < 0);
        o.storq[i] = T;
    }
}

void wallContacts(Oracle& o, double dt)  // calInfiniteWallForceTorque (integrate.cu:514-610)
{
    if (o.nw == 0) return;
#pragma omp parallel for
    for (int i = 0; i < o.ns; ++i) {
        if (o.sdum[i] == 1 || o.sinvm[i] < 1.e-10) continue;
        const double ri = o.srad[i];
        const V3 pi = o.spos[i], vi = o.svel[i], wi = o.sw[i];
        for (int k = 0; k < o.nw; ++k) {
            const int h = i * o.nw + k;
            const V3 n = o.wn[k];
            const double delta = ri - dot(pi - o.wp[k], n);
            if (delta < 0.) {
                o.wslide[h] = o.wroll[h] = o.wtors[h] = mk(0, 0, 0);
                if (o.fixes & DEMSPH_FIX_WALL_LOOP) continue;
                break;
            }
            const double m = 1. / o.sinvm[i];
            const V3 rc = pi - (ri - delta) * n;
            const V3 vc = vi + cross(wi, rc - pi);
            V3 F = mk(0, 0, 0), T = mk(0, 0, 0);
            V3 es = o.wslide[h], er = o.wroll[h], et = o.wtors[h];
            const int c = o.tab.slot(o.smat[i], o.wmat[k]);
            contactLaw(o.tab, c, F, T, es, er, et, vc, wi, n, delta, m, ri, dt);
            o.wslide[h] = es;
            o.wroll[h] = er;
            o.wtors[h] = et;
            o.sacc[i] += F * o.sinvm[i];
            o.storq[i] += T + cross(rc - pi, F);
        }
    }
}

void clumpForce(Oracle& o)  // calClumpForceTorque (integrate.cu:860-881)
{
#pragma omp parallel for
    for (int c = 0; c < o.nc; ++c) {
        V3 F = mk(0, 0, 0), T = mk(0, 0, 0);
        for (int i = o.cstart[c]; i < o.cend[c]; ++i) {
            V3 Fi = mk(0, 0, 0);
            if (o.sinvm[i] > 1.e-10) Fi = o.sacc[i] / o.sinvm[i];
            F += Fi;
            T += o.storq[i] + cross(o.spos[i] - o.cpos[c], Fi);
            o.sacc[i] = mk(0, 0, 0);
            o.storq[i] = mk(0, 0, 0);
        }
        o.cacc[c] = F * o.cinvm[c] + o.g * double(o.cinvm[c] > 0.);
        o.ctorq[c] = T;
    }
}

void solidKick(Oracle& o, double dt)  // solidVelocityAngularVelocityIntegrate (integrate.cu:883-897)
{
#pragma omp parallel for
    for (int i = 0; i < o.ns; ++i) {
        if (o.sclump[i] >= 0) continue;
        o.svel[i] += o.sacc[i] * dt;
        const double r = o.srad[i], im = o.sinvm[i];
        if (im < 1.e-10 || r < 1.e-10) continue;
        const double I = 0.4 * r * r / im;
        o.sw[i] += o.storq[i] / I * dt;
    }
}
void solidDrift(Oracle& o, double dt)  // solidPositionIntegrate (integrate.cu:899-906)
{
#pragma omp parallel for
    for (int i = 0; i < o.ns; ++i) o.spos[i] += dt * o.svel[i];
}
// clumpVelocityAngularVelocityIntegrate (integrate.cu:908-929).
void clumpKick(Oracle& o, double dt)
{
#pragma omp parallel for
    for (int c = 0; c < o.nc; ++c) {
        const V3 a = o.cacc[c], w0 = o.cw[c];
        o.cvel[c] += a * dt;
        if (o.cinvm[c] > 0.) o.cw[c] += (mul(rotateInverseInertia(o.cq[c], o.cinvI[c]), o.ctorq[c])) * dt;
        const V3 w = o.cw[c];
        for (int i = o.cstart[c]; i < o.cend[c]; ++i) {
            const V3 r = o.spos[i] - o.cpos[c];
            o.sacc[i] = a + cross(a, r) + cross(w, cross(w, r));
            o.svel[i] = o.cvel[c] + cross(w, r);
            o.sw[i] = w;
            o.snorm[i] = rotate(o.snorm[i], 0.5 * (w0 + w) * dt);
        }
        if (o.fixes & DEMSPH_FIX_CLUMP_ROTATION) o.cq[c] = quatRotate(o.cq[c], 0.5 * (w0 + w), dt);
    }
}
void clumpDrift(Oracle& o, double dt)  // clumpPositionIntegrate (integrate.cu:931-938)
{
#pragma omp parallel for
    for (int c = 0; c < o.nc; ++c) o.cpos[c] += dt * o.cvel[c];
}

void contactPhase(Oracle& o, double dt)  // calSolidContactAfterFluidIntegrate (integrate.cu:940-962)
{
    pairContacts(o, dt);
    bondContacts(o, dt);
    solidForceGather(o);
    wallContacts(o, dt);
    clumpForce(o);
}
void beforeContact(Oracle& o, double dt)  // solidIntegrateBeforeContact (integrate.cu:964-980)
{
    solidKick(o, 0.5 * dt);
    clumpKick(o, 0.5 * dt);
    clumpDrift(o, 0.5 * dt);
    solidDrift(o, 0.5 * dt);
}
void afterContact(Oracle& o, double dt)  // solidIntegrateAfterContact (integrate.cu:982-998)
{
    solidDrift(o, 0.5 * dt);
    clumpDrift(o, 0.5 * dt);
    clumpKick(o, 0.5 * dt);
    solidKick(o, 0.5 * dt);
}

// addBondData at initialisation (core/dataBase.cpp:270-308): bonds for
// touching same-cluster pairs of the solid list whose bond modulus is set.
// Bonds between touching spheres of one cluster (addBondData,
// core/dataBase.cpp:270-346); after the start only pairs whose first solid is
// above `above` (the last bonded one) are considered.
void addBonds(Oracle& o, int above = -1)
{
    for (int k = 0; k < o.ss.num(); ++k) {
        const int i = o.ss.pointed[k], j = o.ss.pointing[k];
        if (i <= above) continue;
        const V3 pi = o.spos[i], pj = o.spos[j];
        const double ri = o.srad[i], rj = o.srad[j];
        if (ri + rj + 1.e-10 <= len(pi - pj)) continue;
        const int c = o.tab.slot(o.smat[i], o.smat[j]);
        const double Eb = o.tab.bd[6 * c + 1];
        if (Eb > 1.e-10 && o.sclu[i] >= 0 && o.sclu[i] == o.sclu[j]) {
            const double d = len(pi - pj);
            const V3 n = (pi - pj) / d;
            const double delta = ri + rj - d;
            o.bA.push_back(i);
            o.bB.push_back(j);
            o.bOn.push_back(1);
            o.bFn.push_back(0);
            o.bTt.push_back(0);
            o.bFs.push_back(mk(0, 0, 0));
            o.bTb.push_back(mk(0, 0, 0));
            o.bN.push_back(n);
            o.bP.push_back(pj + (rj - 0.5 * delta) * n);
        }
    }
}

// Wendland gradient used for wall normals (core/dataBase.h:262-273).
inline V3 gradWendlandNormal(V3 rij, double h) { return gradWendland(rij, h); }

// setSolidNormal (core/dataBase.cpp:348-413): normals of fixed particles and
// clump pebbles from the kernel gradient of their fixed / same-clump
// neighbours.  With no fluid the reference dereferences max_element of an
// empty range; here the smoothing length is then 0 and all normals are 0.
void setNormals(Oracle& o)
{
    double h = 0;
    for (int i = 0; i < o.nf; ++i) h = std::max(h, o.fh[i]);
    const Grid& G = o.grid;
#pragma omp parallel for
    for (int a = 0; a < o.ns; ++a) {
        V3 th = mk(0, 0, 0);
        const V3 pa = o.spos[a];
        const int ca = o.sclump[a];
        const double ima = o.sinvm[a];
        forStencil(G, pa, [&](int hh) {
            const int st = o.scell.start[hh];
            if (st == -1) return;
            for (int k = st; k < o.scell.end[hh]; ++k) {
                const int b = o.scell.index[k];
                const V3 rab = pa - o.spos[b];
                if (len(rab) > 2 * h) continue;
                if (ima <= 1.e-10 && o.sinvm[b] <= 1.e-10) {
                    const double VB = std::pow(h / 1.3, 3);
                    th += -VB * gradWendlandNormal(rab, h);
                } else if (ca >= 0 && ca == o.sclump[b]) {
                    const double VB = std::pow(2. * o.srad[b], 3.);
                    th += -VB * gradWendlandNormal(rab, h);
                }
            }
        });
        o.snorm[a] = len(th) > 1.e-10 ? unit(th) : mk(0, 0, 0);
    }
}

template <class T>
long copyOut(const T* src, long count, void* out, long cap)
{
    if (out && src && count > 0) std::memcpy(out, src, sizeof(T) * (size_t)std::min(count, cap));
    return count;
}

}  // namespace

extern "C" {

void oracle_set_threads(int n)
{
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

int oracle_max_threads()
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void* oracle_create(const demsph_scene* s, int fixes)
{
    if (!s) return nullptr;
    Oracle* o = new Oracle();
    o->fixes = fixes;
    o->g = mk(s->gravity[0], s->gravity[1], s->gravity[2]);
    o->nf = s->n_fluid;
    o->fpos.resize(o->nf);
    o->fvel.resize(o->nf);
    o->facc.resize(o->nf);
    o->fh.resize(o->nf);
    o->rho0.resize(o->nf);
    o->drho.resize(o->nf);
    o->cs.resize(o->nf);
    o->nu.resize(o->nf);
    o->sumW0.assign(o->nf, 0.);
    for (int i = 0; i < o->nf; ++i) {
        o->fpos[i] = at3(s->fluid_position, i);
        o->fvel[i] = at3(s->fluid_velocity, i);
        o->facc[i] = at3(s->fluid_acceleration, i);
        o->fh[i] = s->fluid_smoothing_length[i];
        o->rho0[i] = s->fluid_rho0[i];
        o->drho[i] = s->fluid_drho ? s->fluid_drho[i] : 0.;
        o->cs[i] = s->fluid_sound_speed[i];
        o->nu[i] = s->fluid_nu[i];
    }
    o->ns = s->n_solid;
    const int ns = o->ns;
    o->spos.resize(ns); o->svel.resize(ns); o->sacc.resize(ns); o->snorm.resize(ns); o->storq.resize(ns);
    o->sw.resize(ns); o->seff.resize(ns); o->srad.resize(ns); o->sinvm.resize(ns); o->smat.resize(ns);
    o->sclu.resize(ns); o->sclump.resize(ns); o->sdum.resize(ns);
    for (int i = 0; i < ns; ++i) {
        o->spos[i] = at3(s->solid_position, i);
        o->svel[i] = at3(s->solid_velocity, i);
        o->sacc[i] = at3(s->solid_acceleration, i);
        o->snorm[i] = at3(s->solid_normal, i);
        o->storq[i] = at3(s->solid_torque, i);
        o->sw[i] = at3(s->solid_angular_velocity, i);
        o->seff[i] = s->solid_effective_radius[i];
        o->srad[i] = s->solid_radius[i];
        o->sinvm[i] = s->solid_inverse_mass[i];
        o->smat[i] = s->solid_material[i];
        o->sclu[i] = s->solid_cluster[i];
        o->sclump[i] = s->solid_clump[i];
        o->sdum[i] = s->solid_is_dummy[i];
    }
    o->nc = s->n_clump;
    const int nc = o->nc;
    o->cpos.resize(nc); o->cvel.resize(nc); o->cacc.resize(nc); o->cw.resize(nc); o->ctorq.resize(nc);
    o->cq.resize(nc); o->cinvI.resize(nc); o->cinvm.resize(nc); o->cstart.resize(nc); o->cend.resize(nc);
    for (int c = 0; c < nc; ++c) {
        o->cpos[c] = at3(s->clump_centroid, c);
        o->cvel[c] = at3(s->clump_velocity, c);
        o->cacc[c] = at3(s->clump_acceleration, c);
        o->cw[c] = at3(s->clump_angular_velocity, c);
        o->ctorq[c] = at3(s->clump_torque, c);
        const double* q = s->clump_orientation + 4 * c;
        o->cq[c] = Quat{q[0], q[1], q[2], q[3]};
        const double* I = s->clump_inverse_inertia + 6 * c;
        o->cinvI[c] = Sym{I[0], I[1], I[2], I[3], I[4], I[5]};
        o->cinvm[c] = s->clump_inverse_mass[c];
        o->cstart[c] = s->clump_pebble_start[c];
        o->cend[c] = s->clump_pebble_end[c];
    }
    o->nw = s->n_wall;
    for (int k = 0; k < o->nw; ++k) {
        o->wp.push_back(at3(s->wall_point, k));
        o->wn.push_back(at3(s->wall_normal, k));
        o->wmat.push_back(s->wall_material[k]);
    }
    o->wslide.assign((size_t)ns * o->nw, mk(0, 0, 0));
    o->wroll = o->wslide;
    o->wtors = o->wslide;
    o->tab.nMat = s->n_material;
    const int nslot = s->n_material * (s->n_material + 1) / 2;
    o->tab.hz.assign(s->hertzian, s->hertzian + 8 * nslot);
    o->tab.ln.assign(s->linear, s->linear + 11 * nslot);
    o->tab.bd.assign(s->bonded, s->bonded + 6 * nslot);
    for (int a = 0; a < 3; ++a) {
        o->domOrg[a] = s->domain_origin[a];
        o->domSize[a] = s->domain_size[a];
    }
    setGrid(*o, *s);
    return o;
}

void oracle_destroy(void* h) { delete static_cast<Oracle*>(h); }

// Device part of solverBase::initialize (core/solverBase.cpp:29-31).
void oracle_initialize(void* h)
{
    Oracle& o = *static_cast<Oracle*>(h);
    neighborSearch(o, 0, 1);
    addBonds(o);
    setNormals(o);
}

// Particles added after the start (dataBase::addFluidData / addSolidData
// with iStep > 0, core/dataBase.cpp:226-268, and addCluster's search and
// bonds, :83-113, :307-343), as the engine's demsph_append does it: the new
// particles follow the old ones in index order with their given state; the
// grid is recomputed; wall springs start from zero (the reference rebuilds
// solid2InfiniteWall); new solids have zero normals; the lists are searched
// at once (the contact springs remapped from the last list); a new cluster is
// bonded above the last bonded solid; new fluids take their Shepard reference
// sums now.  Walls and clumps cannot be added: returns 1 and leaves the state.
int oracle_append(void* h, const demsph_scene* a)
{
    Oracle& o = *static_cast<Oracle*>(h);
    if (!a || a->n_clump != 0 || a->n_wall != 0 || (a->n_fluid <= 0 && a->n_solid <= 0)) return 1;
    for (int i = 0; i < a->n_solid; ++i)
        if (a->solid_material[i] < 0 || a->solid_material[i] >= o.tab.nMat) return 1;
    const int nf0 = o.nf;
    for (int i = 0; i < a->n_fluid; ++i) {
        o.fpos.push_back(at3(a->fluid_position, i));
        o.fvel.push_back(at3(a->fluid_velocity, i));
        o.facc.push_back(at3(a->fluid_acceleration, i));
        o.fh.push_back(a->fluid_smoothing_length[i]);
        o.rho0.push_back(a->fluid_rho0[i]);
        o.drho.push_back(a->fluid_drho ? a->fluid_drho[i] : 0.);
        o.cs.push_back(a->fluid_sound_speed[i]);
        o.nu.push_back(a->fluid_nu[i]);
        o.sumW0.push_back(0.);
    }
    o.nf += a->n_fluid;
    bool cluster = false;
    for (int i = 0; i < a->n_solid; ++i) {
        o.spos.push_back(at3(a->solid_position, i));
        o.svel.push_back(at3(a->solid_velocity, i));
        o.sacc.push_back(at3(a->solid_acceleration, i));
        o.snorm.push_back(mk(0, 0, 0));
        o.storq.push_back(at3(a->solid_torque, i));
        o.sw.push_back(at3(a->solid_angular_velocity, i));
        o.seff.push_back(a->solid_effective_radius[i]);
        o.srad.push_back(a->solid_radius[i]);
        o.sinvm.push_back(a->solid_inverse_mass[i]);
        o.smat.push_back(a->solid_material[i]);
        o.sclu.push_back(a->solid_cluster ? a->solid_cluster[i] : -1);
        o.sclump.push_back(-1);
        o.sdum.push_back(a->solid_is_dummy ? a->solid_is_dummy[i] : 0);
        cluster |= o.sclu.back() >= 0;
    }
    o.ns += a->n_solid;
    o.wslide.assign((size_t)o.ns * o.nw, mk(0, 0, 0));
    o.wroll = o.wslide;
    o.wtors = o.wslide;
    demsph_scene dom{};
    for (int k = 0; k < 3; ++k) {
        dom.domain_origin[k] = o.domOrg[k];
        dom.domain_size[k] = o.domSize[k];
    }
    setGrid(o, dom);
    neighborSearch(o, 0, 1);
    if (cluster) addBonds(o, o.bA.empty() ? -1 : o.bA.back());
    for (int i = nf0; i < o.nf; ++i) o.sumW0[i] = shepardSum(o, i);
    return 0;
}

void oracle_neighbor_search(void* h, int iStep, int gap) { neighborSearch(*static_cast<Oracle*>(h), iStep, gap); }
void oracle_solid_integrate_before_contact(void* h, double dt) { beforeContact(*static_cast<Oracle*>(h), dt); }
void oracle_fluid_integrate(void* h, double dt, int iStep, int gap)
{
    fluidIntegrate(*static_cast<Oracle*>(h), dt, iStep, gap);
}
void oracle_solid_contact_after_fluid_integrate(void* h, double dt) { contactPhase(*static_cast<Oracle*>(h), dt); }
void oracle_solid_integrate_after_contact(void* h, double dt) { afterContact(*static_cast<Oracle*>(h), dt); }

// solverBase::update (core/solverBase.cpp:47-58) for n consecutive steps.
void oracle_update(void* h, double dt, int firstStep, int nSteps, int gap)
{
    Oracle& o = *static_cast<Oracle*>(h);
    for (int s = firstStep; s < firstStep + nSteps; ++s) {
        neighborSearch(o, s, gap);
        beforeContact(o, dt);
        fluidIntegrate(o, dt, s, gap);
        contactPhase(o, dt);
        afterContact(o, dt);
    }
}

// Same array names as oracle/ref_harness.cpp's ref_get.
long oracle_get(void* h, const char* name, void* out, long cap)
{
    Oracle& o = *static_cast<Oracle*>(h);
    const std::string s(name);
    const long nf = o.nf, ns = o.ns, nc = o.nc;
    auto v3 = [&](const std::vector<V3>& v) { return copyOut(v.empty() ? nullptr : &v[0].x, 3 * (long)v.size(), out, cap) / 3; };
    auto vi = [&](const std::vector<int>& v) { return copyOut(v.empty() ? nullptr : v.data(), (long)v.size(), out, cap); };
    auto vd = [&](const std::vector<double>& v) { return copyOut(v.empty() ? nullptr : v.data(), (long)v.size(), out, cap); };
    const Grid& G = o.grid;
    if (s == "grid.num") return G.num;
    if (s == "grid.gridSize") { int g3[3] = {G.gx, G.gy, G.gz}; return copyOut(g3, 3, out, cap); }
    if (s == "grid.minBound") return copyOut(&G.minB.x, 3, out, cap);
    if (s == "grid.maxBound") return copyOut(&G.maxB.x, 3, out, cap);
    if (s == "grid.cellSize") return copyOut(&G.cs.x, 3, out, cap);
    if (s == "grid.cellStartFluid") return vi(o.fcell.start);
    if (s == "grid.cellEndFluid") return vi(o.fcell.end);
    if (s == "grid.cellStartSolid") return vi(o.scell.start);
    if (s == "grid.cellEndSolid") return vi(o.scell.end);
    if (s == "fluid.pos") return v3(o.fpos);
    if (s == "fluid.vel") return v3(o.fvel);
    if (s == "fluid.acc") return v3(o.facc);
    if (s == "fluid.h") return vd(o.fh);
    if (s == "fluid.dRho") return vd(o.drho);
    if (s == "fluid.sumW0") return vd(o.sumW0);
    if (s == "fluid.hash.value") return vi(o.fcell.value);
    if (s == "fluid.hash.index") return vi(o.fcell.index);
    if (s == "fluid.ffPrefix") return vi(o.ff.prefix);
    if (s == "fluid.fsPrefix") return vi(o.fs.prefix);
    if (s == "fluid.fluidRange.start") return vi(o.ff.rev.start);
    if (s == "fluid.fluidRange.end") return vi(o.ff.rev.end);
    if (s == "solid.pos") return v3(o.spos);
    if (s == "solid.vel") return v3(o.svel);
    if (s == "solid.acc") return v3(o.sacc);
    if (s == "solid.angvel") return v3(o.sw);
    if (s == "solid.torque") return v3(o.storq);
    if (s == "solid.normal") return v3(o.snorm);
    if (s == "solid.radius") return vd(o.srad);
    if (s == "solid.effRadius") return vd(o.seff);
    if (s == "solid.invMass") return vd(o.sinvm);
    if (s == "solid.hash.value") return vi(o.scell.value);
    if (s == "solid.hash.index") return vi(o.scell.index);
    if (s == "solid.ssPrefix") return vi(o.ss.prefix);
    if (s == "solid.solidRange.start") return vi(o.ss.rev.start);
    if (s == "solid.solidRange.end") return vi(o.ss.rev.end);
    if (s == "solid.fluidSolidRange.start") return vi(o.fs.rev.start);
    if (s == "solid.fluidSolidRange.end") return vi(o.fs.rev.end);
    if (s == "clump.centroid") return v3(o.cpos);
    if (s == "clump.vel") return v3(o.cvel);
    if (s == "clump.acc") return v3(o.cacc);
    if (s == "clump.angvel") return v3(o.cw);
    if (s == "clump.torque") return v3(o.ctorq);
    if (s == "clump.orientation")  // q0 q1 q2 q3 per clump
        return copyOut(o.cq.empty() ? nullptr : &o.cq[0].q0, 4 * (long)o.cq.size(), out, cap) / 4;
    if (s == "ff.pointed") return vi(o.ff.pointed);
    if (s == "ff.pointing") return vi(o.ff.pointing);
    if (s == "ff.hash.index") return vi(o.ff.rev.index);
    if (s == "fs.pointed") return vi(o.fs.pointed);
    if (s == "fs.pointing") return vi(o.fs.pointing);
    if (s == "fs.force") return v3(o.fsForce);
    if (s == "fs.hash.index") return vi(o.fs.rev.index);
    if (s == "ss.pointed") return vi(o.ss.pointed);
    if (s == "ss.pointing") return vi(o.ss.pointing);
    if (s == "ss.force") return v3(o.ssF);
    if (s == "ss.torque") return v3(o.ssT);
    if (s == "ss.sliding") return v3(o.ssS);
    if (s == "ss.rolling") return v3(o.ssR);
    if (s == "ss.torsion") return v3(o.ssTo);
    if (s == "ss.hash.index") return vi(o.ss.rev.index);
    if (s == "bond.pointed") return vi(o.bA);
    if (s == "bond.pointing") return vi(o.bB);
    if (s == "bond.isBonded") return vi(o.bOn);
    if (s == "bond.normalForce") return vd(o.bFn);
    if (s == "bond.torsionTorque") return vd(o.bTt);
    if (s == "bond.shearForce") return v3(o.bFs);
    if (s == "bond.bendingTorque") return v3(o.bTb);
    if (s == "bond.contactNormal") return v3(o.bN);
    if (s == "bond.contactPoint") return v3(o.bP);
    (void)nf; (void)ns; (void)nc;
    return -1;
}

}  // extern "C"
