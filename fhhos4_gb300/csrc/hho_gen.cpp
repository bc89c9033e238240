// Host-side producer of the multigrid hierarchy the solve phase consumes: the statically
// condensed HHO face system A_l, right-hand side b and prolongations P_l of fhhos4's
// geometric h-multigrid, for the in-house meshes of the unit square (2 triangles per cell)
// and the unit cube (6 tetrahedra per cube).
//
// It reproduces the reference's discretisation so that the system is the reference's own
// (up to rounding):
//   * mesh numbering: Square_TriangularMesh::Build (src/Mesher/InHouse/Square_TriangularMesh.h:113-233),
//     Cube_CartesianTetrahedralMesh::Build (src/Mesher/InHouse/Cube_CartesianTetrahedralMesh.h:24-104),
//     faces renumbered interior-first (src/Mesh/Mesh.h:331-340);
//   * standard coarsening links (Square_TriangularMesh.h:368-400, Cube_CartesianTetrahedralMesh.h:120-162,
//     Mesh.h:696-732);
//   * face bases: Legendre on edges (2D), monomials in the face's reference coordinates
//     orthogonalised once by Gram-Schmidt (3D) (src/Discretizations/HHO/Diff_HHOFace.h:55-70,
//     src/FunctionalBasis/Orthogonal/OrthogonalBasis.h:96-114);
//   * HHO reconstruction, "hho" stabilisation, static condensation and condensed RHS
//     (src/Discretizations/HHO/Diff_HHOElement.h:303-470, Diffusion_HHO.h:600-640);
//   * prolongation P = Pi_f I_c with heterogeneous face weights and R = P^T
//     (src/Solver/Multigrid/MultigridForHHO/LevelForHHO.h:182-213,743-954).
// Cell bases are this file's own (orthonormalised scaled monomials): the condensed operator
// and P do not depend on that choice. Integrals are exact (collapsed Gauss-Legendre rules)
// except the source term, integrated with a high-order rule.
#include "hho_gen.h"

#include <algorithm>
#include <array>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <functional>
#include <string>
#include <thread>
#include <unordered_map>
#include <map>
#include <vector>

namespace {

constexpr double kPi = 3.14159265358979323846;

// ---------------------------------------------------------------------------
// Small dense helpers (row-major)

struct Mat {
    int r = 0, c = 0;
    std::vector<double> a;
    Mat() {}
    Mat(int r_, int c_) : r(r_), c(c_), a((size_t)r_ * c_, 0.0) {}
    double& operator()(int i, int j) { return a[(size_t)i * c + j]; }
    double operator()(int i, int j) const { return a[(size_t)i * c + j]; }
};

Mat matmul(const Mat& A, const Mat& B)
{
    Mat C(A.r, B.c);
    for (int i = 0; i < A.r; i++)
        for (int k = 0; k < A.c; k++) {
            const double v = A(i, k);
            if (v == 0.0) continue;
            for (int j = 0; j < B.c; j++) C(i, j) += v * B(k, j);
        }
    return C;
}

Mat transpose(const Mat& A)
{
    Mat T(A.c, A.r);
    for (int i = 0; i < A.r; i++)
        for (int j = 0; j < A.c; j++) T(j, i) = A(i, j);
    return T;
}

// Solve A X = B (A square) by LU with partial pivoting; returns false if singular.
bool solve(Mat A, Mat& B)
{
    const int n = A.r;
    std::vector<int> piv(n);
    for (int k = 0; k < n; k++) {
        int p = k;
        for (int i = k + 1; i < n; i++)
            if (std::fabs(A(i, k)) > std::fabs(A(p, k))) p = i;
        if (A(p, k) == 0.0) return false;
        if (p != k) {
            for (int j = 0; j < n; j++) std::swap(A(k, j), A(p, j));
            for (int j = 0; j < B.c; j++) std::swap(B(k, j), B(p, j));
        }
        for (int i = k + 1; i < n; i++) {
            const double f = A(i, k) / A(k, k);
            if (f == 0.0) continue;
            for (int j = k; j < n; j++) A(i, j) -= f * A(k, j);
            for (int j = 0; j < B.c; j++) B(i, j) -= f * B(k, j);
        }
    }
    for (int i = n - 1; i >= 0; i--)
        for (int j = 0; j < B.c; j++) {
            double v = B(i, j);
            for (int k = i + 1; k < n; k++) v -= A(i, k) * B(k, j);
            B(i, j) = v / A(i, i);
        }
    return true;
}

// ---------------------------------------------------------------------------
// Quadrature: Gauss-Legendre on [0,1] and collapsed rules on the reference simplex.

void gauss_legendre01(int m, std::vector<double>& x, std::vector<double>& w)
{
    x.resize(m);
    w.resize(m);
    for (int i = 0; i < m; i++) {
        long double z = std::cos(kPi * (i + 0.75L) / (m + 0.5L)), pp = 0;
        for (int it = 0; it < 100; it++) {
            long double p1 = 1, p2 = 0;
            for (int j = 1; j <= m; j++) {
                const long double p3 = p2;
                p2 = p1;
                p1 = ((2 * j - 1) * z * p2 - (j - 1) * p3) / j;
            }
            pp = m * (z * p1 - p2) / (z * z - 1);
            const long double dz = p1 / pp;
            z -= dz;
            if (std::fabs((double)dz) < 1e-19) break;
        }
        x[i] = (double)((1 - z) / 2);
        w[i] = (double)(1 / ((1 - z * z) * pp * pp));
    }
}

struct RefRule {
    std::vector<std::array<double, 3>> p;  // reference simplex coordinates
    std::vector<double> w;                 // weights summing to the reference measure
};

// Exact for polynomials of degree <= 2m-1-(dim-1) on the reference simplex.
RefRule simplex_rule(int dim, int m)
{
    std::vector<double> x, w;
    gauss_legendre01(m, x, w);
    RefRule R;
    if (dim == 1) {
        for (int i = 0; i < m; i++) { R.p.push_back({x[i], 0, 0}); R.w.push_back(w[i]); }
    } else if (dim == 2) {
        for (int i = 0; i < m; i++)
            for (int j = 0; j < m; j++) {
                const double a = x[i], b = x[j];
                R.p.push_back({a * (1 - b), b, 0});
                R.w.push_back(w[i] * w[j] * (1 - b));
            }
    } else {
        for (int i = 0; i < m; i++)
            for (int j = 0; j < m; j++)
                for (int k = 0; k < m; k++) {
                    const double a = x[i], b = x[j], c = x[k];
                    R.p.push_back({a * (1 - b) * (1 - c), b * (1 - c), c});
                    R.w.push_back(w[i] * w[j] * w[k] * (1 - b) * (1 - c) * (1 - c));
                }
    }
    return R;
}

// ---------------------------------------------------------------------------
// Meshes

struct Mesh {
    int dim = 2, n = 0;
    std::vector<std::array<double, 3>> vx;
    std::vector<std::array<int, 4>> el;        // vertices (dim+1)
    std::vector<std::array<int, 3>> fv;        // face vertices in the face's own order (dim)
    std::vector<int> fe1, fe2;                 // face elements (fe2 = -1 on the boundary)
    std::vector<std::array<int, 4>> ef;        // element faces (dim+1)
    std::vector<int> efn;                      // faces added so far per element (build only)
    std::vector<int> interior_order;           // faces in the order they became interior
    std::vector<int> number;                   // face -> unknown block (-1: Dirichlet face)
    int n_interior = 0;
    std::vector<int> coarser;                  // element -> coarser element (standard coarsening)
    std::vector<int> removed;                  // face -> 1 if interior to a coarse element
    std::vector<std::array<double, 9>> K;      // diffusion tensor per element (row-major dim x dim)
};

void add_face_to_element(Mesh& M, int e, int f) { M.ef[e][M.efn[e]++] = f; }

void finalize_numbering(Mesh& M)
{
    M.number.assign(M.fv.size(), -1);
    int k = 0;
    for (int f : M.interior_order) M.number[f] = k++;
    M.n_interior = k;
}

Mesh build_tri(int n)
{
    Mesh M;
    M.dim = 2; M.n = n;
    const double h = 1.0 / n;
    for (int iy = 0; iy <= n; iy++)
        for (int ix = 0; ix <= n; ix++) M.vx.push_back({ix * h, iy * h, 0.0});
    auto V = [&](int ix, int iy) { return iy * (n + 1) + ix; };
    auto E = [&](int ix, int iy) { return (iy * n + ix) * 2; };
    M.el.resize((size_t)2 * n * n);
    for (int iy = 0; iy < n; iy++)
        for (int ix = 0; ix < n; ix++) {
            const int bl = V(ix, iy), tl = V(ix, iy + 1), tr = V(ix + 1, iy + 1), br = V(ix + 1, iy);
            M.el[E(ix, iy)] = {bl, br, tl, -1};       // lower (V1, V2, V3)
            M.el[E(ix, iy) + 1] = {tl, br, tr, -1};   // upper
        }
    M.ef.assign(M.el.size(), {-1, -1, -1, -1});
    M.efn.assign(M.el.size(), 0);
    auto face = [&](int a, int b, int e1, int e2) {
        const int f = (int)M.fv.size();
        M.fv.push_back({a, b, -1});
        M.fe1.push_back(e1);
        M.fe2.push_back(e2);
        add_face_to_element(M, e1, f);
        if (e2 >= 0) { add_face_to_element(M, e2, f); M.interior_order.push_back(f); }
        return f;
    };
    for (int ix = 0; ix < n; ix++) {
        const int lo = E(ix, 0);
        face(M.el[lo][0], M.el[lo][1], lo, -1);                 // south: lower V1-V2
        const int up = E(ix, n - 1) + 1;
        face(M.el[up][0], M.el[up][2], up, -1);                 // north: upper V1-V3
    }
    for (int iy = 0; iy < n; iy++) {
        const int lo = E(0, iy);
        face(M.el[lo][2], M.el[lo][0], lo, -1);                 // west: lower V3-V1
        const int up = E(n - 1, iy) + 1;
        face(M.el[up][1], M.el[up][2], up, -1);                 // east: upper V2-V3
    }
    for (int iy = 0; iy < n; iy++)
        for (int ix = 0; ix < n; ix++) {
            const int lo = E(ix, iy), up = lo + 1;
            face(M.el[lo][2], M.el[lo][1], lo, up);              // diagonal: lower V3-V2
            if (ix != n - 1) {
                const int ea = E(ix + 1, iy);
                face(M.el[ea][2], M.el[ea][0], up, ea);          // east neighbour V3-V1
            }
            if (iy != n - 1) {
                const int no = E(ix, iy + 1);
                face(M.el[no][0], M.el[no][1], up, no);          // north neighbour V1-V2
            }
        }
    finalize_numbering(M);
    return M;
}

struct TriKey {
    int a, b, c;
    bool operator==(const TriKey& o) const { return a == o.a && b == o.b && c == o.c; }
};
struct TriKeyHash {
    size_t operator()(const TriKey& k) const
    {
        return ((size_t)k.a * 73856093u) ^ ((size_t)k.b * 19349663u) ^ ((size_t)k.c * 83492791u);
    }
};

Mesh build_tet(int n)
{
    Mesh M;
    M.dim = 3; M.n = n;
    const double h = 1.0 / n;
    for (int iz = 0; iz <= n; iz++)
        for (int iy = 0; iy <= n; iy++)
            for (int ix = 0; ix <= n; ix++) M.vx.push_back({ix * h, iy * h, iz * h});
    auto V = [&](int ix, int iy, int iz) { return (iz * (n + 1) + iy) * (n + 1) + ix; };
    const size_t ne = (size_t)6 * n * n * n;
    M.el.reserve(ne);
    M.ef.assign(ne, {-1, -1, -1, -1});
    M.efn.assign(ne, 0);
    std::unordered_map<TriKey, int, TriKeyHash> lookup;
    lookup.reserve((size_t)14 * n * n * n);
    auto key = [](int a, int b, int c) {
        int v[3] = {a, b, c};
        std::sort(v, v + 3);
        return TriKey{v[0], v[1], v[2]};
    };
    auto new_face = [&](int a, int b, int c, int e1, int e2) {
        const int f = (int)M.fv.size();
        M.fv.push_back({a, b, c});
        M.fe1.push_back(e1);
        M.fe2.push_back(e2);
        return f;
    };
    // CreateFaceIfNeeded (TetrahedralMesh.h:263-283)
    auto face_if_needed = [&](int e, int a, int b, int c) {
        auto k = key(a, b, c);
        auto it = lookup.find(k);
        int f;
        if (it == lookup.end()) {
            f = new_face(a, b, c, e, -1);
            lookup.emplace(k, f);
        } else {
            f = it->second;
            M.fe2[f] = e;
            M.interior_order.push_back(f);
        }
        add_face_to_element(M, e, f);
    };
    // CreateInteriorFace (TetrahedralMesh.h:285-299)
    auto interior_face = [&](int e1, int e2, int a, int b, int c) {
        const int f = new_face(a, b, c, e1, e2);
        lookup.emplace(key(a, b, c), f);
        M.interior_order.push_back(f);
        add_face_to_element(M, e1, f);
        add_face_to_element(M, e2, f);
    };
    for (int iz = 0; iz < n; iz++)
        for (int iy = 0; iy < n; iy++)
            for (int ix = 0; ix < n; ix++) {
                const int v000 = V(ix, iy, iz), v100 = V(ix + 1, iy, iz), v110 = V(ix + 1, iy + 1, iz),
                          v111 = V(ix + 1, iy + 1, iz + 1), v101 = V(ix + 1, iy, iz + 1), v010 = V(ix, iy + 1, iz),
                          v011 = V(ix, iy + 1, iz + 1), v001 = V(ix, iy, iz + 1);
                const int t0 = (int)M.el.size();
                M.el.push_back({v010, v110, v111, v100});
                M.el.push_back({v111, v010, v100, v000});
                M.el.push_back({v000, v100, v111, v101});
                M.el.push_back({v111, v010, v000, v011});
                M.el.push_back({v101, v111, v000, v011});
                M.el.push_back({v101, v000, v001, v011});
                const int t1 = t0 + 1, t2 = t0 + 2, t3 = t0 + 3, t4 = t0 + 4, t5 = t0 + 5;
                face_if_needed(t0, v010, v111, v110);
                face_if_needed(t0, v010, v110, v100);
                interior_face(t0, t1, v010, v100, v111);
                face_if_needed(t0, v100, v110, v111);
                interior_face(t1, t3, v111, v010, v000);
                interior_face(t1, t2, v111, v000, v100);
                face_if_needed(t1, v000, v010, v100);
                face_if_needed(t2, v000, v100, v101);
                interior_face(t2, t4, v000, v101, v111);
                face_if_needed(t2, v101, v100, v111);
                face_if_needed(t3, v111, v010, v011);
                interior_face(t3, t4, v111, v011, v000);
                face_if_needed(t3, v011, v010, v000);
                face_if_needed(t4, v101, v111, v011);
                interior_face(t4, t5, v101, v011, v000);
                face_if_needed(t5, v101, v001, v000);
                face_if_needed(t5, v101, v011, v001);
                face_if_needed(t5, v011, v000, v001);
            }
    finalize_numbering(M);
    return M;
}

std::array<double, 3> centroid(const Mesh& M, int e)
{
    std::array<double, 3> c{0, 0, 0};
    for (int i = 0; i <= M.dim; i++)
        for (int d = 0; d < 3; d++) c[d] += M.vx[M.el[e][i]][d];
    for (int d = 0; d < 3; d++) c[d] /= (M.dim + 1);
    return c;
}

double simplex_volume(const Mesh& M, const std::array<double, 3>* P, int dim)
{
    if (dim == 2) {
        return 0.5 * std::fabs((P[1][0] - P[0][0]) * (P[2][1] - P[0][1]) - (P[2][0] - P[0][0]) * (P[1][1] - P[0][1]));
    }
    double a[3], b[3], c[3];
    for (int d = 0; d < 3; d++) { a[d] = P[1][d] - P[0][d]; b[d] = P[2][d] - P[0][d]; c[d] = P[3][d] - P[0][d]; }
    const double det = a[0] * (b[1] * c[2] - b[2] * c[1]) - a[1] * (b[0] * c[2] - b[2] * c[0]) + a[2] * (b[0] * c[1] - b[1] * c[0]);
    (void)M;
    return std::fabs(det) / 6.0;
}

// Tetrahedron/Triangle::Contains: barycentric coordinates from sub-volumes, tolerance 1e-4
// (src/Geometry/3D/Tetrahedron.h:147-161, Utils::Eps).
bool contains(const Mesh& M, int e, const std::array<double, 3>& p)
{
    const int nv = M.dim + 1;
    std::array<double, 3> P[4];
    for (int i = 0; i < nv; i++) P[i] = M.vx[M.el[e][i]];
    const double vol = simplex_volume(M, P, M.dim);
    const double tol = 1e-4;
    double sum = 0;
    for (int i = 0; i < nv; i++) {
        std::array<double, 3> Q[4];
        for (int j = 0; j < nv; j++) Q[j] = P[j];
        Q[i] = p;
        const double l = simplex_volume(M, Q, M.dim) / vol;
        if (!(l + tol > 0 && l < 1 + tol)) return false;
        sum += l;
    }
    return std::fabs(sum - 1) < tol;
}

// Standard coarsening links: fine element -> coarse element containing its centre, searched
// among the coarse simplices of the coarse cell that holds the fine cell.
void link_coarse(Mesh& F, const Mesh& C)
{
    const int per = F.dim == 2 ? 2 : 6;
    F.coarser.assign(F.el.size(), -1);
    const int n = F.n, nc = C.n;
    for (size_t e = 0; e < F.el.size(); e++) {
        const int cell = (int)(e / per);
        int ix, iy, iz = 0;
        if (F.dim == 2) { ix = cell % n; iy = cell / n; }
        else { ix = cell % n; iy = (cell / n) % n; iz = cell / (n * n); }
        const int ccell = F.dim == 2 ? (iy / 2) * nc + ix / 2 : ((iz / 2) * nc + iy / 2) * nc + ix / 2;
        const auto c = centroid(F, (int)e);
        for (int j = 0; j < per; j++) {
            const int ce = ccell * per + j;
            if (contains(C, ce, c)) { F.coarser[e] = ce; break; }
        }
    }
    F.removed.assign(F.fv.size(), 0);
    for (size_t f = 0; f < F.fv.size(); f++)
        if (F.fe2[f] >= 0) F.removed[f] = F.coarser[F.fe1[f]] == F.coarser[F.fe2[f]];
}

// ---------------------------------------------------------------------------
// Polynomial spaces

// Exponents of the monomials of total degree <= p, ordered by degree.
std::vector<std::array<int, 3>> exponents(int dim, int p)
{
    std::vector<std::array<int, 3>> ex;
    for (int deg = 0; deg <= p; deg++) {
        if (dim == 1) ex.push_back({deg, 0, 0});
        else if (dim == 2)
            for (int j = 0; j <= deg; j++) ex.push_back({deg - j, j, 0});
        else
            for (int c = 0; c <= deg; c++)
                for (int b = 0; b <= deg - c; b++) ex.push_back({deg - b - c, b, c});
    }
    return ex;
}

double ipow(double x, int k)
{
    double r = 1;
    for (int i = 0; i < k; i++) r *= x;
    return r;
}

double legendre(int n, double x)
{
    if (n == 0) return 1;
    if (n == 1) return x;
    double p0 = 1, p1 = x;
    for (int j = 2; j <= n; j++) {
        const double p2 = ((2 * j - 1) * x * p1 - (j - 1) * p0) / j;
        p0 = p1;
        p1 = p2;
    }
    return p1;
}

// Cell basis: scaled monomials ((x - xT)/hT)^alpha orthonormalised in L2(T) (two sweeps).
struct CellBasis {
    int dim = 0, nR = 0;
    std::vector<std::array<int, 3>> ex;
    std::array<double, 3> xc{0, 0, 0};
    double hs = 1;
    Mat coef;  // nR x nR: phi_i = sum_j coef(i,j) m_j
    void eval_monomials(const double* x, double* m, double* gm /* nR x 3 or null */) const
    {
        eval_monomials_at(x, xc.data(), m, gm);
    }
    // The same basis translated to centre c (elements of one class differ by a translation).
    void eval_monomials_at(const double* x, const double* c, double* m, double* gm) const
    {
        double y[3] = {0, 0, 0};
        for (int d = 0; d < dim; d++) y[d] = (x[d] - c[d]) / hs;
        for (int j = 0; j < nR; j++) {
            const auto& e = ex[j];
            m[j] = ipow(y[0], e[0]) * ipow(y[1], e[1]) * ipow(y[2], e[2]);
            if (gm) {
                for (int d = 0; d < 3; d++) {
                    double g = 0;
                    if (d < dim && e[d] > 0) {
                        g = e[d] / hs;
                        for (int q = 0; q < 3; q++) g *= ipow(y[q], e[q] - (q == d ? 1 : 0));
                    }
                    gm[j * 3 + d] = g;
                }
            }
        }
    }
    void eval(const double* x, double* v, double* g) const { eval_at(x, xc.data(), v, g); }
    // Values of the first `count` basis functions only (the basis is hierarchical: phi_i combines
    // monomials 0..i), centred at c.
    void eval_first_at(const double* x, const double* c, int count, double* v) const
    {
        double y[3] = {0, 0, 0};
        for (int d = 0; d < dim; d++) y[d] = (x[d] - c[d]) / hs;
        double m[64];
        for (int j = 0; j < count; j++) {
            const auto& e = ex[j];
            m[j] = ipow(y[0], e[0]) * ipow(y[1], e[1]) * ipow(y[2], e[2]);
        }
        for (int i = 0; i < count; i++) {
            double s = 0;
            for (int j = 0; j <= i; j++) s += coef(i, j) * m[j];
            v[i] = s;
        }
    }
    void eval_at(const double* x, const double* c, double* v, double* g) const
    {
        double m[64], gm[192];
        eval_monomials_at(x, c, m, g ? gm : nullptr);
        for (int i = 0; i < nR; i++) {
            double s = 0, gx = 0, gy = 0, gz = 0;
            for (int j = 0; j <= i; j++) {
                const double c = coef(i, j);
                s += c * m[j];
                if (g) { gx += c * gm[j * 3]; gy += c * gm[j * 3 + 1]; gz += c * gm[j * 3 + 2]; }
            }
            v[i] = s;
            if (g) { g[i * 3] = gx; g[i * 3 + 1] = gy; g[i * 3 + 2] = gz; }
        }
    }
};

// Physical quadrature points of an element / face.
struct QPts {
    std::vector<std::array<double, 3>> x;
    std::vector<std::array<double, 2>> ref;  // face reference coordinates (t[, u])
    std::vector<double> w;
};

struct Rules {
    RefRule cell, cell_rhs, face;
};

QPts element_points(const Mesh& M, int e, const RefRule& R)
{
    QPts Q;
    const int dim = M.dim;
    const auto& X0 = M.vx[M.el[e][0]];
    double J[3][3] = {{0}};
    for (int c = 0; c < dim; c++)
        for (int d = 0; d < dim; d++) J[d][c] = M.vx[M.el[e][c + 1]][d] - X0[d];
    double det;
    if (dim == 2) det = J[0][0] * J[1][1] - J[0][1] * J[1][0];
    else
        det = J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) - J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
              J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
    det = std::fabs(det);
    for (size_t q = 0; q < R.w.size(); q++) {
        std::array<double, 3> x{0, 0, 0};
        for (int d = 0; d < dim; d++) {
            x[d] = X0[d];
            for (int c = 0; c < dim; c++) x[d] += J[d][c] * R.p[q][c];
        }
        Q.x.push_back(x);
        Q.w.push_back(R.w[q] * det);
    }
    return Q;
}

// Face points in the face's own reference coordinates: 2D edges t in [-1,1] with
// x = (v2-v1)/2 t + (v2+v1)/2 (src/Geometry/2D/Segment.h:117-128); 3D triangles
// x = v1 + (v2-v1) t + (v3-v1) u (src/Geometry/3D/TriangleIn3D.h:152-162).
QPts face_points(const Mesh& M, int f, const RefRule& R1, const RefRule& R2, double& measure, double& diameter)
{
    QPts Q;
    if (M.dim == 2) {
        const auto& a = M.vx[M.fv[f][0]];
        const auto& b = M.vx[M.fv[f][1]];
        const double len = std::hypot(b[0] - a[0], b[1] - a[1]);
        measure = diameter = len;
        for (size_t q = 0; q < R1.w.size(); q++) {
            const double t = 2 * R1.p[q][0] - 1;  // [0,1] -> [-1,1]
            Q.x.push_back({(b[0] - a[0]) / 2 * t + (b[0] + a[0]) / 2, (b[1] - a[1]) / 2 * t + (b[1] + a[1]) / 2, 0});
            Q.ref.push_back({t, 0});
            Q.w.push_back(R1.w[q] * len);
        }
    } else {
        const auto& a = M.vx[M.fv[f][0]];
        const auto& b = M.vx[M.fv[f][1]];
        const auto& c = M.vx[M.fv[f][2]];
        double ab[3], ac[3], bc[3];
        for (int d = 0; d < 3; d++) { ab[d] = b[d] - a[d]; ac[d] = c[d] - a[d]; bc[d] = c[d] - b[d]; }
        const double cr[3] = {ab[1] * ac[2] - ab[2] * ac[1], ab[2] * ac[0] - ab[0] * ac[2], ab[0] * ac[1] - ab[1] * ac[0]};
        measure = 0.5 * std::sqrt(cr[0] * cr[0] + cr[1] * cr[1] + cr[2] * cr[2]);
        auto nrm = [](const double* v) { return std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]); };
        diameter = std::max({nrm(ab), nrm(ac), nrm(bc)});
        for (size_t q = 0; q < R2.w.size(); q++) {
            const double t = R2.p[q][0], u = R2.p[q][1];
            Q.x.push_back({a[0] + ab[0] * t + ac[0] * u, a[1] + ab[1] * t + ac[1] * u, a[2] + ab[2] * t + ac[2] * u});
            Q.ref.push_back({t, u});
            Q.w.push_back(R2.w[q] * 2 * measure);
        }
    }
    return Q;
}

// Reference face basis of one face: values at the face points (nf x nq) and the face mass matrix.
struct FaceBasis {
    int nf = 0;
    Mat vals;  // nf x nq
    Mat mass;  // nf x nf
    Mat mass_inv;
};

FaceBasis face_basis(int dim, int k, const QPts& Q)
{
    FaceBasis B;
    const int nq = (int)Q.w.size();
    if (dim == 2) {
        // LegendreBasis1D, not orthogonalised (src/FunctionalBasis/Legendre/Legendre1D.h:37-45)
        B.nf = k + 1;
        B.vals = Mat(B.nf, nq);
        for (int i = 0; i < B.nf; i++)
            for (int q = 0; q < nq; q++) B.vals(i, q) = legendre(i, Q.ref[q][0]);
    } else {
        // MonomialBasis2D in (t, u), Gram-Schmidt once, not normalised (OrthogonalBasis.h:96-114)
        auto ex = exponents(2, k);
        B.nf = (int)ex.size();
        B.vals = Mat(B.nf, nq);
        std::vector<double> norm2(B.nf);
        for (int i = 0; i < B.nf; i++) {
            for (int q = 0; q < nq; q++) B.vals(i, q) = ipow(Q.ref[q][0], ex[i][0]) * ipow(Q.ref[q][1], ex[i][1]);
            for (int j = 0; j < i; j++) {
                double ip = 0;
                for (int q = 0; q < nq; q++) ip += Q.w[q] * B.vals(i, q) * B.vals(j, q);
                const double c = ip / norm2[j];
                for (int q = 0; q < nq; q++) B.vals(i, q) -= c * B.vals(j, q);
            }
            double n2 = 0;
            for (int q = 0; q < nq; q++) n2 += Q.w[q] * B.vals(i, q) * B.vals(i, q);
            norm2[i] = n2;
        }
    }
    B.mass = Mat(B.nf, B.nf);
    for (int i = 0; i < B.nf; i++)
        for (int j = 0; j < B.nf; j++) {
            double s = 0;
            for (int q = 0; q < nq; q++) s += Q.w[q] * B.vals(i, q) * B.vals(j, q);
            B.mass(i, j) = s;
        }
    if (dim == 3) {
        // orthogonal basis: the reference applies diag(NormSquare)
        for (int i = 0; i < B.nf; i++)
            for (int j = 0; j < B.nf; j++)
                if (i != j) B.mass(i, j) = 0.0;
    }
    B.mass_inv = Mat(B.nf, B.nf);
    for (int i = 0; i < B.nf; i++) B.mass_inv(i, i) = 1.0;
    solve(B.mass, B.mass_inv);
    return B;
}

// ---------------------------------------------------------------------------
// Element operators

struct ElementOps {
    CellBasis basis;
    int nC = 0, nR = 0, nf = 0, nF = 0;
    Mat P;       // nR x (nC + nF nf) reconstruction
    Mat A;       // (nC + nF nf)^2 local operator
    Mat schur;   // (nF nf)^2 condensed
    Mat solve_cells;  // nC x nF nf: -A_TT^{-1} A_TF
    Mat interp;  // nR x nF nf: P [solve_cells; I] (ReconstructionFromFacesMatrix)
    std::vector<double> bT;    // nC: (f, c_j)_T
    std::vector<double> bF;    // nF nf: condensed RHS contribution
    std::vector<double> cell_rhs;  // nC: A_TT^{-1} b_T (cell unknowns = cell_rhs + solve_cells x_F)
    Mat att_inv;  // nC x nC: A_TT^{-1}, for the source terms of the elements of this one's class
    Mat atf;      // nC x nF nf: A_TF
    Mat local;    // (nC + nF nf)^2: the local operator before condensation (cells first, then faces)
    bool ok = true;
};

struct Params {
    int dim, k;
    int source;  // 0: d pi^2 prod sin(pi x_i); 1: 1; 2: four random sine modes
    double amp[4] = {0, 0, 0, 0};   // source 2: f = sum_i amp_i prod_d sin(pi m_id x_d)
    int mode[4][3] = {};
};

double source_value(const Params& p, const std::array<double, 3>& x)
{
    if (p.source == 1) return 1.0;
    if (p.source == 2) {
        double f = 0.0;
        for (int i = 0; i < 4; i++) {
            double t = p.amp[i];
            for (int d = 0; d < p.dim; d++) t *= std::sin(kPi * p.mode[i][d] * x[d]);
            f += t;
        }
        return f;
    }
    if (p.dim == 2) return 2 * kPi * kPi * std::sin(kPi * x[0]) * std::sin(kPi * x[1]);
    return 3 * kPi * kPi * std::sin(kPi * x[0]) * std::sin(kPi * x[1]) * std::sin(kPi * x[2]);
}

// Outward unit normal of face f of element e.
std::array<double, 3> outer_normal(const Mesh& M, int e, int f)
{
    std::array<double, 3> n{0, 0, 0};
    const auto& a = M.vx[M.fv[f][0]];
    const auto& b = M.vx[M.fv[f][1]];
    if (M.dim == 2) {
        n = {b[1] - a[1], -(b[0] - a[0]), 0};
    } else {
        const auto& c = M.vx[M.fv[f][2]];
        const double ab[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]}, ac[3] = {c[0] - a[0], c[1] - a[1], c[2] - a[2]};
        n = {ab[1] * ac[2] - ab[2] * ac[1], ab[2] * ac[0] - ab[0] * ac[2], ab[0] * ac[1] - ab[1] * ac[0]};
    }
    const double len = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
    for (auto& v : n) v /= len;
    const auto ce = centroid(M, e);
    double s = 0;
    for (int d = 0; d < 3; d++) s += n[d] * (a[d] - ce[d]);
    if (s < 0)
        for (auto& v : n) v = -v;
    return n;
}

void Kgrad(const std::array<double, 9>& K, int dim, const double* g, double* out)
{
    for (int i = 0; i < 3; i++) out[i] = 0;
    for (int i = 0; i < dim; i++)
        for (int j = 0; j < dim; j++) out[i] += K[i * dim + j] * g[j];
}

double nKn(const std::array<double, 9>& K, int dim, const std::array<double, 3>& n)
{
    double s = 0;
    for (int i = 0; i < dim; i++)
        for (int j = 0; j < dim; j++) s += n[i] * K[i * dim + j] * n[j];
    return s;
}

ElementOps element_ops(const Mesh& M, int e, const Params& prm, const Rules& rules, bool want_interp)
{
    ElementOps O;
    const int dim = M.dim, k = prm.k;
    const auto& K = M.K[e];
    CellBasis& B = O.basis;
    B.dim = dim;
    B.ex = exponents(dim, k + 1);
    B.nR = (int)B.ex.size();
    B.xc = centroid(M, e);
    double hmax = 0;
    for (int i = 0; i <= dim; i++)
        for (int j = i + 1; j <= dim; j++) {
            double s = 0;
            for (int d = 0; d < 3; d++) s += std::pow(M.vx[M.el[e][i]][d] - M.vx[M.el[e][j]][d], 2);
            hmax = std::max(hmax, std::sqrt(s));
        }
    B.hs = hmax;
    O.nR = B.nR;
    O.nC = (int)exponents(dim, k).size();
    O.nF = dim + 1;
    const QPts QE = element_points(M, e, rules.cell);
    const int nq = (int)QE.w.size();
    // Orthonormalise the scaled monomials (modified Gram-Schmidt, two sweeps).
    {
        Mat mv(B.nR, nq);
        double m[64];
        for (int q = 0; q < nq; q++) {
            B.eval_monomials(QE.x[q].data(), m, nullptr);
            for (int j = 0; j < B.nR; j++) mv(j, q) = m[j];
        }
        B.coef = Mat(B.nR, B.nR);
        Mat vals(B.nR, nq);
        for (int i = 0; i < B.nR; i++) {
            B.coef(i, i) = 1.0;
            for (int q = 0; q < nq; q++) vals(i, q) = mv(i, q);
            for (int sweep = 0; sweep < 2; sweep++)
                for (int j = 0; j < i; j++) {
                    double ip = 0;
                    for (int q = 0; q < nq; q++) ip += QE.w[q] * vals(i, q) * vals(j, q);
                    for (int q = 0; q < nq; q++) vals(i, q) -= ip * vals(j, q);
                    for (int c = 0; c <= j; c++) B.coef(i, c) -= ip * B.coef(j, c);
                }
            double n2 = 0;
            for (int q = 0; q < nq; q++) n2 += QE.w[q] * vals(i, q) * vals(i, q);
            const double inv = 1.0 / std::sqrt(n2);
            for (int q = 0; q < nq; q++) vals(i, q) *= inv;
            for (int c = 0; c <= i; c++) B.coef(i, c) *= inv;
        }
    }
    const int nR = O.nR, nC = O.nC;
    // Stiffness S and mean values.
    Mat S(nR, nR);
    std::vector<double> mean(nR, 0.0);
    {
        double v[64], g[192], kg[3];
        for (int q = 0; q < nq; q++) {
            B.eval(QE.x[q].data(), v, g);
            for (int i = 0; i < nR; i++) {
                mean[i] += QE.w[q] * v[i];
                Kgrad(K, dim, &g[i * 3], kg);
                for (int j = 0; j < nR; j++) S(i, j) += QE.w[q] * (kg[0] * g[j * 3] + kg[1] * g[j * 3 + 1] + kg[2] * g[j * 3 + 2]);
            }
        }
    }
    // Faces: points, bases, normals.
    struct FaceData { QPts Q; FaceBasis FB; std::array<double, 3> n; double measure, diam; Mat cellvals; Mat gradn; };
    std::vector<FaceData> FD(O.nF);
    for (int lf = 0; lf < O.nF; lf++) {
        const int f = M.ef[e][lf];
        FaceData& D = FD[lf];
        D.Q = face_points(M, f, rules.face, rules.face, D.measure, D.diam);
        D.FB = face_basis(dim, k, D.Q);
        D.n = outer_normal(M, e, f);
        const int nfq = (int)D.Q.w.size();
        D.cellvals = Mat(nR, nfq);
        D.gradn = Mat(nR, nfq);
        double v[64], g[192], kg[3];
        for (int q = 0; q < nfq; q++) {
            B.eval(D.Q.x[q].data(), v, g);
            for (int i = 0; i < nR; i++) {
                D.cellvals(i, q) = v[i];
                Kgrad(K, dim, &g[i * 3], kg);
                D.gradn(i, q) = kg[0] * D.n[0] + kg[1] * D.n[1] + kg[2] * D.n[2];
            }
        }
    }
    O.nf = FD[0].FB.nf;
    const int nf = O.nf, nF = O.nF, nH = nC + nF * nf;
    // Reconstruction: [S L; L^T 0] [P; lambda] = [rhs; mean condition]
    Mat sys(nR + 1, nR + 1), rhs(nR + 1, nH);
    for (int i = 0; i < nR; i++) {
        for (int j = 0; j < nR; j++) sys(i, j) = S(i, j);
        sys(i, nR) = mean[i];
        sys(nR, i) = mean[i];
    }
    for (int i = 0; i < nR; i++) {
        for (int j = 0; j < nC; j++) {
            double v = S(i, j);  // hierarchical orthonormal basis: c_j = r_j
            for (int lf = 0; lf < nF; lf++) {
                const FaceData& D = FD[lf];
                for (size_t q = 0; q < D.Q.w.size(); q++) v -= D.Q.w[q] * D.gradn(i, q) * D.cellvals(j, q);
            }
            rhs(i, j) = v;
        }
        for (int lf = 0; lf < nF; lf++) {
            const FaceData& D = FD[lf];
            for (int a = 0; a < nf; a++) {
                double v = 0;
                for (size_t q = 0; q < D.Q.w.size(); q++) v += D.Q.w[q] * D.gradn(i, q) * D.FB.vals(a, q);
                rhs(i, nC + lf * nf + a) = v;
            }
        }
    }
    for (int j = 0; j < nC; j++) rhs(nR, j) = mean[j];
    if (!solve(sys, rhs)) { O.ok = false; return O; }
    O.P = Mat(nR, nH);
    for (int i = 0; i < nR; i++)
        for (int j = 0; j < nH; j++) O.P(i, j) = rhs(i, j);
    // Consistency: P^T S P.
    Mat Acons = matmul(transpose(O.P), matmul(S, O.P));
    // Stabilisation (Diff_HHOElement.h:378-413).
    Mat Astab(nH, nH);
    Mat Dt(nC, nH);
    for (int i = 0; i < nC; i++)
        for (int j = 0; j < nH; j++) Dt(i, j) = O.P(i, j) - (i == j ? 1.0 : 0.0);
    for (int lf = 0; lf < nF; lf++) {
        const FaceData& D = FD[lf];
        const int nfq = (int)D.Q.w.size();
        Mat tr(nf, nR);  // M_F^{-1} (phi_a, r_j)_F
        {
            Mat m(nf, nR);
            for (int a = 0; a < nf; a++)
                for (int j = 0; j < nR; j++) {
                    double s = 0;
                    for (int q = 0; q < nfq; q++) s += D.Q.w[q] * D.FB.vals(a, q) * D.cellvals(j, q);
                    m(a, j) = s;
                }
            tr = matmul(D.FB.mass_inv, m);
        }
        Mat Df = matmul(tr, O.P);
        for (int a = 0; a < nf; a++) Df(a, nC + lf * nf + a) -= 1.0;
        Mat trT(nf, nC);
        for (int a = 0; a < nf; a++)
            for (int j = 0; j < nC; j++) trT(a, j) = tr(a, j);
        Mat diff = matmul(trT, Dt);
        for (int a = 0; a < nf; a++)
            for (int j = 0; j < nH; j++) diff(a, j) = Df(a, j) - diff(a, j);
        const double coeff = nKn(K, dim, D.n) / D.diam;
        Mat md = matmul(D.FB.mass, diff);
        for (int i = 0; i < nH; i++)
            for (int j = 0; j < nH; j++) {
                double s = 0;
                for (int a = 0; a < nf; a++) s += diff(a, i) * md(a, j);
                Astab(i, j) += s * coeff;
            }
    }
    O.A = Mat(nH, nH);
    for (size_t i = 0; i < O.A.a.size(); i++) O.A.a[i] = Acons.a[i] + Astab.a[i];
    O.local = O.A;
    // Static condensation.
    const int nFF = nF * nf;
    Mat Att(nC, nC), Atf(nC, nFF);
    for (int i = 0; i < nC; i++) {
        for (int j = 0; j < nC; j++) Att(i, j) = O.A(i, j);
        for (int j = 0; j < nFF; j++) Atf(i, j) = O.A(i, nC + j);
    }
    // RHS (f, c_j)_T with a high-order rule.
    O.bT.assign(nC, 0.0);
    {
        const QPts QR = element_points(M, e, rules.cell_rhs);
        double v[64];
        for (size_t q = 0; q < QR.w.size(); q++) {
            B.eval(QR.x[q].data(), v, nullptr);
            const double fv = source_value(prm, QR.x[q]);
            for (int j = 0; j < nC; j++) O.bT[j] += QR.w[q] * fv * v[j];
        }
    }
    Mat X = Atf;  // A_TT^{-1} A_TF
    Mat rhsb(nC, 1);
    for (int j = 0; j < nC; j++) rhsb(j, 0) = O.bT[j];
    O.att_inv = Mat(nC, nC);
    for (int j = 0; j < nC; j++) O.att_inv(j, j) = 1.0;
    if (!solve(Att, X) || !solve(Att, rhsb) || !solve(Att, O.att_inv)) { O.ok = false; return O; }
    O.atf = Atf;
    O.schur = Mat(nFF, nFF);
    for (int i = 0; i < nFF; i++)
        for (int j = 0; j < nFF; j++) {
            double s = O.A(nC + i, nC + j);
            for (int c = 0; c < nC; c++) s -= Atf(c, i) * X(c, j);
            O.schur(i, j) = s;
        }
    O.cell_rhs.assign(nC, 0.0);
    for (int c = 0; c < nC; c++) O.cell_rhs[c] = rhsb(c, 0);
    O.bF.assign(nFF, 0.0);
    for (int i = 0; i < nFF; i++) {
        double s = 0;
        for (int c = 0; c < nC; c++) s += Atf(c, i) * rhsb(c, 0);
        O.bF[i] = -s;
    }
    if (want_interp) {
        O.solve_cells = Mat(nC, nFF);
        for (int i = 0; i < nC; i++)
            for (int j = 0; j < nFF; j++) O.solve_cells(i, j) = -X(i, j);
        Mat H(nH, nFF);
        for (int i = 0; i < nC; i++)
            for (int j = 0; j < nFF; j++) H(i, j) = O.solve_cells(i, j);
        for (int j = 0; j < nFF; j++) H(nC + j, j) = 1.0;
        O.interp = matmul(O.P, H);
        O.A = Mat();
    } else {
        O.P = Mat();
        O.A = Mat();
    }
    return O;
}

// ---------------------------------------------------------------------------
// Parallel loop

void parallel_for(size_t n, int threads, const std::function<void(size_t, size_t)>& body)
{
    if (threads <= 1 || n < 256) { body(0, n); return; }
    std::vector<std::thread> th;
    std::atomic<size_t> next{0};
    const size_t chunk = std::max<size_t>(64, n / (threads * 16));
    for (int t = 0; t < threads; t++)
        th.emplace_back([&]() {
            for (;;) {
                const size_t s = next.fetch_add(chunk);
                if (s >= n) break;
                body(s, std::min(n, s + chunk));
            }
        });
    for (auto& t : th) t.join();
}

// ---------------------------------------------------------------------------
// Levels

struct Level {
    Mesh mesh;
    // Element-local operators per class of elements that differ only by a translation (same vertex
    // offsets, same face vertex orders, same diffusion tensor): the local matrices depend on nothing
    // else, because every cell basis is centred on its element. The source term does depend on the
    // position, so the condensed right-hand side and the cell part of the RHS are kept per element.
    std::vector<ElementOps> cls_ops;
    std::vector<int> cls;                 // element -> class
    std::vector<double> bF_e;             // per element, nF nf: condensed RHS contribution (finest level)
    std::vector<double> cell_rhs_e;       // per element, nC: A_TT^{-1} b_T (finest level)
    std::vector<double> bT_e;             // per element, nC: b_T = (f, c_j)_T (finest level)
    std::vector<double> cls_local;        // per class, the local operator before condensation (kept
    int cls_nC = 0, cls_nFF = 0;          // when cls_ops is released), its cell and face unknowns
    int n_rows = 0;
    std::vector<int> A_rowptr, A_colidx;
    std::vector<double> A_vals;
    std::vector<double> b;
    std::vector<int> P_rowptr, P_colidx;
    std::vector<double> P_vals;
    int P_cols = 0;
    // Tables of P (kept when asked for, fhg_hho_prolongation_tables): per unknown fine face its
    // coarse elements (up to two, -1: none), their weights and contribution slots; per slot the
    // nf x (dim + 1) nf contribution of a coarse element to a fine face.
    std::vector<int> Pt_ce, Pt_slot;
    std::vector<double> Pt_w, Pt_contrib;
    int Pt_nslots = 0;
};

// What element_ops depends on besides the element's position: the offsets of its vertices and of
// every local face's vertices (in the face's own order, which fixes the face basis) from its first
// vertex, in units of the mesh spacing h rounded to h / 4096, and the bits of its diffusion tensor.
std::vector<long long> element_key(const Mesh& M, int e, double h)
{
    const int dim = M.dim;
    std::vector<long long> key;
    key.reserve(32);
    const auto& v0 = M.vx[M.el[e][0]];
    auto put = [&](int vi) {
        for (int d = 0; d < dim; d++) key.push_back(std::llround((M.vx[vi][d] - v0[d]) / h * 4096.0));
    };
    for (int i = 1; i <= dim; i++) put(M.el[e][i]);
    for (int lf = 0; lf <= dim; lf++)
        for (int j = 0; j < dim; j++) put(M.fv[M.ef[e][lf]][j]);
    for (int i = 0; i < 9; i++) {
        long long bits;
        std::memcpy(&bits, &M.K[e][i], sizeof(bits));
        key.push_back(bits);
    }
    return key;
}

// The source terms of element e with its class's local operators O: b_T = (f, c_j)_T on the element's
// own quadrature points and centred basis, cell_rhs = A_TT^{-1} b_T, bF = -A_FT A_TT^{-1} b_T.
void element_rhs(const Mesh& M, int e, const Params& prm, const Rules& rules, const ElementOps& O, double* bF,
                 double* cell_rhs, double* bT_out)
{
    const int nC = O.nC, nFF = O.nF * O.nf;
    const auto xc = centroid(M, e);
    double bT[64] = {0};
    const QPts QR = element_points(M, e, rules.cell_rhs);
    double v[64];
    for (size_t q = 0; q < QR.w.size(); q++) {
        O.basis.eval_first_at(QR.x[q].data(), xc.data(), nC, v);
        const double fv = source_value(prm, QR.x[q]);
        for (int j = 0; j < nC; j++) bT[j] += QR.w[q] * fv * v[j];
    }
    for (int j = 0; j < nC; j++) bT_out[j] = bT[j];
    for (int c = 0; c < nC; c++) {
        double s = 0;
        for (int j = 0; j < nC; j++) s += O.att_inv(c, j) * bT[j];
        cell_rhs[c] = s;
    }
    for (int i = 0; i < nFF; i++) {
        double s = 0;
        for (int c = 0; c < nC; c++) s += O.atf(c, i) * cell_rhs[c];
        bF[i] = -s;
    }
}

// Element classes of a level, their local operators (computed once per class, in parallel), and on
// the finest level every element's source terms.
int element_classes(Level& L, const Params& prm, const Rules& rules, int threads, bool finest)
{
    const Mesh& M = L.mesh;
    const size_t ne = M.el.size();
    const double h = 1.0 / M.n;
    std::vector<std::vector<long long>> keys(ne);
    parallel_for(ne, threads, [&](size_t s, size_t e) {
        for (size_t i = s; i < e; i++) keys[i] = element_key(M, (int)i, h);
    });
    std::map<std::vector<long long>, int> index;
    std::vector<int> reps;
    L.cls.assign(ne, 0);
    for (size_t i = 0; i < ne; i++) {
        auto it = index.find(keys[i]);
        if (it == index.end()) {
            it = index.emplace(std::move(keys[i]), (int)reps.size()).first;
            reps.push_back((int)i);
        }
        L.cls[i] = it->second;
    }
    std::vector<std::vector<long long>>().swap(keys);
    L.cls_ops.assign(reps.size(), ElementOps());
    std::atomic<int> bad{0};
    parallel_for(reps.size(), threads, [&](size_t s, size_t e) {
        for (size_t c = s; c < e; c++) {
            L.cls_ops[c] = element_ops(M, reps[c], prm, rules, true);
            if (!L.cls_ops[c].ok) bad++;
        }
    });
    if (bad) return -2;
    if (finest) {
        const int nC = L.cls_ops[0].nC, nFF = L.cls_ops[0].nF * L.cls_ops[0].nf;
        L.bF_e.assign(ne * nFF, 0.0);
        L.cell_rhs_e.assign(ne * nC, 0.0);
        L.bT_e.assign(ne * nC, 0.0);
        parallel_for(ne, threads, [&](size_t s, size_t e) {
            for (size_t i = s; i < e; i++)
                element_rhs(M, (int)i, prm, rules, L.cls_ops[L.cls[i]], &L.bF_e[i * nFF], &L.cell_rhs_e[i * nC],
                            &L.bT_e[i * nC]);
        });
    }
    return 0;
}

// Global condensed operator and RHS of one level.
void assemble(Level& L, const Params& prm, int threads, bool want_rhs)
{
    Mesh& M = L.mesh;
    const int nf = (int)L.cls_ops[0].nf, nF = M.dim + 1;
    const int nI = M.n_interior;
    L.n_rows = nI * nf;
    // Block pattern: faces of the elements of each interior face.
    std::vector<std::array<int, 8>> cols(nI);
    std::vector<int> ncols(nI, 0);
    std::vector<int> face_of(nI);
    for (size_t f = 0; f < M.fv.size(); f++)
        if (M.number[f] >= 0) face_of[M.number[f]] = (int)f;
    parallel_for(nI, threads, [&](size_t s, size_t e) {
        for (size_t I = s; I < e; I++) {
            const int f = face_of[I];
            std::array<int, 8> c;
            int nc = 0;
            for (int side = 0; side < 2; side++) {
                const int el = side == 0 ? M.fe1[f] : M.fe2[f];
                for (int lf = 0; lf < nF; lf++) {
                    const int g = M.number[M.ef[el][lf]];
                    if (g < 0) continue;
                    bool seen = false;
                    for (int q = 0; q < nc; q++) seen |= c[q] == g;
                    if (!seen) c[nc++] = g;
                }
            }
            std::sort(c.begin(), c.begin() + nc);
            cols[I] = c;
            ncols[I] = nc;
        }
    });
    L.A_rowptr.assign((size_t)L.n_rows + 1, 0);
    for (int I = 0; I < nI; I++)
        for (int a = 0; a < nf; a++) L.A_rowptr[(size_t)I * nf + a + 1] = ncols[I] * nf;
    for (int r = 0; r < L.n_rows; r++) L.A_rowptr[r + 1] += L.A_rowptr[r];
    L.A_colidx.assign(L.A_rowptr[L.n_rows], 0);
    L.A_vals.assign(L.A_rowptr[L.n_rows], 0.0);
    if (want_rhs) L.b.assign(L.n_rows, 0.0);
    parallel_for(nI, threads, [&](size_t s, size_t e) {
        for (size_t I = s; I < e; I++) {
            const int f = face_of[I];
            for (int a = 0; a < nf; a++) {
                const size_t row = (size_t)I * nf + a;
                int p = L.A_rowptr[row];
                for (int q = 0; q < ncols[I]; q++)
                    for (int bb = 0; bb < nf; bb++) L.A_colidx[p++] = cols[I][q] * nf + bb;
            }
            for (int side = 0; side < 2; side++) {
                const int el = side == 0 ? M.fe1[f] : M.fe2[f];
                const ElementOps& O = L.cls_ops[L.cls[el]];
                int lfi = -1;
                for (int lf = 0; lf < nF; lf++)
                    if (M.ef[el][lf] == f) lfi = lf;
                for (int lf = 0; lf < nF; lf++) {
                    const int g = M.number[M.ef[el][lf]];
                    if (g < 0) continue;
                    int q = 0;
                    while (cols[I][q] != g) q++;
                    for (int a = 0; a < nf; a++) {
                        const size_t row = (size_t)I * nf + a;
                        double* dst = &L.A_vals[L.A_rowptr[row] + q * nf];
                        for (int bb = 0; bb < nf; bb++) dst[bb] += O.schur(lfi * nf + a, lf * nf + bb);
                    }
                }
                if (want_rhs)
                    for (int a = 0; a < nf; a++)
                        L.b[(size_t)I * nf + a] += L.bF_e[(size_t)el * nF * nf + lfi * nf + a];
            }
        }
    });
}

// P (fine faces x coarse faces) of LevelForHHO::SetupProlongation_H with CellInterp_Trace; with
// `tables`, also the tables of P (Level::Pt_*).
void prolongation(Level& F, const Level& C, const Params& prm, const Rules& rules, int threads, bool tables)
{
    const Mesh& M = F.mesh;
    const Mesh& MC = C.mesh;
    const int dim = M.dim, nf = C.cls_ops[0].nf, nFc = dim + 1;
    const int nI = M.n_interior;
    std::vector<int> face_of(nI);
    for (size_t f = 0; f < M.fv.size(); f++)
        if (M.number[f] >= 0) face_of[M.number[f]] = (int)f;
    std::vector<std::array<int, 8>> cols(nI);
    std::vector<int> ncols(nI, 0);
    auto coarse_elems = [&](int f, int* ce, double* w, int& nce) {
        const int e1 = M.fe1[f], e2 = M.fe2[f];
        if (M.removed[f]) { ce[0] = M.coarser[e1]; w[0] = 1.0; nce = 1; return; }
        const auto n1 = outer_normal(M, e1, f);
        const auto n2 = outer_normal(M, e2, f);
        const double k1 = nKn(M.K[e1], dim, n1), k2 = nKn(M.K[e2], dim, n2);
        ce[0] = M.coarser[e1]; w[0] = k1 / (k1 + k2);
        ce[1] = M.coarser[e2]; w[1] = k2 / (k1 + k2);
        nce = 2;
    };
    // The contribution of coarse element ce to the fine face of points Q and basis FB:
    // M_f^{-1} (phi_a, r_j)_f (the trace of the coarse reconstruction basis on the fine face) times
    // the coarse element's interpolation from its faces, nf x (nFc nf).
    auto contribution = [&](const QPts& Q, const FaceBasis& FB, int ce) {
        const ElementOps& O = C.cls_ops[C.cls[ce]];
        const auto xc = centroid(MC, ce);
        const int nR = O.nR, nfq = (int)Q.w.size();
        Mat m(nf, nR);
        double v[64];
        for (int q = 0; q < nfq; q++) {
            O.basis.eval_at(Q.x[q].data(), xc.data(), v, nullptr);
            for (int a = 0; a < nf; a++)
                for (int j = 0; j < nR; j++) m(a, j) += Q.w[q] * FB.vals(a, q) * v[j];
        }
        Mat tr = matmul(FB.mass_inv, m);
        return matmul(tr, O.interp);
    };
    parallel_for(nI, threads, [&](size_t s, size_t e) {
        for (size_t I = s; I < e; I++) {
            const int f = face_of[I];
            int ce[2], nce;
            double w[2];
            coarse_elems(f, ce, w, nce);
            std::array<int, 8> c;
            int nc = 0;
            for (int t = 0; t < nce; t++)
                for (int lf = 0; lf < nFc; lf++) {
                    const int g = MC.number[MC.ef[ce[t]][lf]];
                    if (g < 0) continue;
                    bool seen = false;
                    for (int q = 0; q < nc; q++) seen |= c[q] == g;
                    if (!seen) c[nc++] = g;
                }
            std::sort(c.begin(), c.begin() + nc);
            cols[I] = c;
            ncols[I] = nc;
        }
    });
    F.P_cols = C.n_rows;
    F.P_rowptr.assign((size_t)nI * nf + 1, 0);
    for (int I = 0; I < nI; I++)
        for (int a = 0; a < nf; a++) F.P_rowptr[(size_t)I * nf + a + 1] = ncols[I] * nf;
    for (size_t r = 0; r < (size_t)nI * nf; r++) F.P_rowptr[r + 1] += F.P_rowptr[r];
    F.P_colidx.assign(F.P_rowptr.back(), 0);
    F.P_vals.assign(F.P_rowptr.back(), 0.0);
    parallel_for(nI, threads, [&](size_t s, size_t e) {
        for (size_t I = s; I < e; I++) {
            const int f = face_of[I];
            for (int a = 0; a < nf; a++) {
                int p = F.P_rowptr[(size_t)I * nf + a];
                for (int q = 0; q < ncols[I]; q++)
                    for (int bb = 0; bb < nf; bb++) F.P_colidx[p++] = cols[I][q] * nf + bb;
            }
            int ce[2], nce;
            double w[2];
            coarse_elems(f, ce, w, nce);
            double measure, diam;
            const QPts Q = face_points(M, f, rules.face, rules.face, measure, diam);
            const FaceBasis FB = face_basis(dim, prm.k, Q);
            for (int t = 0; t < nce; t++) {
                const Mat contrib = contribution(Q, FB, ce[t]);  // nf x (nFc nf)
                for (int lf = 0; lf < nFc; lf++) {
                    const int g = MC.number[MC.ef[ce[t]][lf]];
                    if (g < 0) continue;
                    int q = 0;
                    while (cols[I][q] != g) q++;
                    for (int a = 0; a < nf; a++) {
                        double* dst = &F.P_vals[F.P_rowptr[(size_t)I * nf + a] + q * nf];
                        for (int bb = 0; bb < nf; bb++) dst[bb] += w[t] * contrib(a, lf * nf + bb);
                    }
                }
            }
        }
    });
    if (!tables) return;
    // A coarse element's contribution to a fine face depends only on the element's class and on
    // where the face lies in it: the face's vertices, in the face's own order (which fixes its
    // basis), relative to the element's first vertex, in units of the fine spacing rounded to 1/4096
    // of it. One slot per such pair, computed once.
    struct KeyHash {
        size_t operator()(const std::array<long long, 10>& k) const
        {
            uint64_t hsh = 1469598103934665603ull;
            for (long long v : k) hsh = (hsh ^ (uint64_t)v) * 1099511628211ull;
            return (size_t)hsh;
        }
    };
    std::unordered_map<std::array<long long, 10>, int, KeyHash> slot_of;
    std::vector<std::pair<int, int>> reps;   // per slot: (fine face, coarse element)
    F.Pt_ce.assign((size_t)nI * 2, -1);
    F.Pt_slot.assign((size_t)nI * 2, -1);
    F.Pt_w.assign((size_t)nI * 2, 0.0);
    const double scale = 4096.0 * M.n;
    for (int I = 0; I < nI; I++) {
        const int f = face_of[I];
        int ce[2], nce;
        double w[2];
        coarse_elems(f, ce, w, nce);
        for (int t = 0; t < nce; t++) {
            std::array<long long, 10> key{};
            key[0] = C.cls[ce[t]];
            const auto& x0 = MC.vx[MC.el[ce[t]][0]];
            for (int v = 0; v < dim; v++)
                for (int d = 0; d < dim; d++) key[1 + v * 3 + d] = std::llround((M.vx[M.fv[f][v]][d] - x0[d]) * scale);
            const auto ins = slot_of.emplace(key, (int)reps.size());
            if (ins.second) reps.emplace_back(f, ce[t]);
            F.Pt_ce[(size_t)I * 2 + t] = ce[t];
            F.Pt_w[(size_t)I * 2 + t] = w[t];
            F.Pt_slot[(size_t)I * 2 + t] = ins.first->second;
        }
    }
    const int ncc = nFc * nf;
    F.Pt_nslots = (int)reps.size();
    F.Pt_contrib.assign((size_t)reps.size() * nf * ncc, 0.0);
    parallel_for(reps.size(), threads, [&](size_t s, size_t e) {
        for (size_t r = s; r < e; r++) {
            double measure, diam;
            const QPts Q = face_points(M, reps[r].first, rules.face, rules.face, measure, diam);
            const FaceBasis FB = face_basis(dim, prm.k, Q);
            const Mat c = contribution(Q, FB, reps[r].second);
            for (int a = 0; a < nf; a++)
                for (int j = 0; j < ncc; j++) F.Pt_contrib[(r * nf + a) * ncc + j] = c(a, j);
        }
    });
}

uint64_t splitmix64(uint64_t& s)
{
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
double uniform01(uint64_t& s) { return (splitmix64(s) >> 11) * (1.0 / 9007199254740992.0); }

// Tensor of one coefficient block (bx, by, bz) of the field: a pure function of the seed and
// the block index, so every level of the hierarchy sees the same field.
std::array<double, 9> block_tensor(const fhg_hho_params& p, int dim, int bx, int by, int bz)
{
    std::array<double, 9> K{0, 0, 0, 0, 0, 0, 0, 0, 0};
    const int m = p.checker_blocks > 0 ? p.checker_blocks : 4;
    uint64_t s = p.seed * 0x100000001B3ull + (uint64_t)((bz * m + by) * m + bx) + 1;
    if (p.coefficient == FHG_HHO_CHECKERBOARD) {
        const double kappa = ((bx + by + bz) % 2 == 0) ? 1.0 : p.contrast;
        for (int i = 0; i < dim; i++) K[i * dim + i] = kappa;
    } else if (p.coefficient == FHG_HHO_LOGNORMAL_PATCHES) {
        const double lc = std::log(p.contrast > 1 ? p.contrast : 1.0);
        const double kappa = std::exp(-lc + 2 * lc * uniform01(s));
        for (int i = 0; i < dim; i++) K[i * dim + i] = kappa;
    } else if (p.coefficient == FHG_HHO_ANISOTROPIC) {
        const double emin = p.eps_min > 0 ? p.eps_min : 1e-3;
        const double eps = std::exp(std::log(emin) * (1.0 - uniform01(s)));
        double R[3][3];
        if (dim == 3) {
            // uniform random rotation from a unit quaternion (Shoemake)
            const double u1 = uniform01(s), u2 = uniform01(s), u3 = uniform01(s);
            const double a = std::sqrt(1 - u1), b = std::sqrt(u1);
            const double q0 = a * std::sin(2 * kPi * u2), q1 = a * std::cos(2 * kPi * u2);
            const double q2 = b * std::sin(2 * kPi * u3), q3 = b * std::cos(2 * kPi * u3);
            const double w = q0, x = q1, y = q2, z = q3;
            R[0][0] = 1 - 2 * (y * y + z * z); R[0][1] = 2 * (x * y - z * w); R[0][2] = 2 * (x * z + y * w);
            R[1][0] = 2 * (x * y + z * w); R[1][1] = 1 - 2 * (x * x + z * z); R[1][2] = 2 * (y * z - x * w);
            R[2][0] = 2 * (x * z - y * w); R[2][1] = 2 * (y * z + x * w); R[2][2] = 1 - 2 * (x * x + y * y);
        } else {
            const double th = 2 * kPi * uniform01(s);
            R[0][0] = std::cos(th); R[0][1] = -std::sin(th); R[1][0] = std::sin(th); R[1][1] = std::cos(th);
        }
        double D[3] = {1, 1, 1};
        D[dim - 1] = eps;
        for (int i = 0; i < dim; i++)
            for (int j = 0; j < dim; j++) {
                double v = 0;
                for (int q = 0; q < dim; q++) v += R[i][q] * D[q] * R[j][q];
                K[i * dim + j] = v;
            }
    } else {
        for (int i = 0; i < dim; i++) K[i * dim + i] = 1.0;
    }
    return K;
}

// Coefficient of every element: the tensor of the block holding its centre (per-element
// tensors keyed on the element centre, on every level).
void set_coefficients(Mesh& M, const fhg_hho_params& p)
{
    const int dim = M.dim;
    const int m = p.checker_blocks > 0 ? p.checker_blocks : 4;
    M.K.assign(M.el.size(), {0, 0, 0, 0, 0, 0, 0, 0, 0});
    for (size_t e = 0; e < M.el.size(); e++) {
        const auto c = centroid(M, (int)e);
        int bi[3] = {0, 0, 0};
        for (int d = 0; d < dim; d++) bi[d] = std::min(m - 1, std::max(0, (int)std::floor(c[d] * m)));
        M.K[e] = block_tensor(p, dim, bi[0], bi[1], bi[2]);
    }
}

}  // namespace

// ===========================================================================

struct fhg_hho {
    std::vector<Level> levels;
    std::string err;
    int block_size = 0;
    Params prm{2, 1, 0};
    Rules rules;
    int threads = 1;
};

extern "C" {

void fhg_hho_default_params(fhg_hho_params* p)
{
    std::memset(p, 0, sizeof(*p));
    p->dim = 3;
    p->n = 8;
    p->k = 1;
    p->max_coarse_rows = 1000;
    p->max_levels = 0;
    p->source = FHG_HHO_SOURCE_SINE;
    p->coefficient = FHG_HHO_IDENTITY;
    p->contrast = 1.0;
    p->checker_blocks = 4;
    p->threads = 0;
    p->eps_min = 1e-3;
    p->seed = 20261203ull;
}

int fhg_hho_create(fhg_hho** out, const fhg_hho_params* p)
{
    if (!out || !p) return -1;
    fhg_hho* H = new fhg_hho();
    *out = H;
    if ((p->dim != 2 && p->dim != 3) || p->n < 1 || p->k < 1 || p->k > 3) {
        H->err = "unsupported dim/n/k (dim 2 or 3, n >= 1, k in 1..3)";
        return -1;
    }
    const int threads = p->threads > 0 ? p->threads : (int)std::max(1u, std::thread::hardware_concurrency());
    Params prm{p->dim, p->k, p->source == FHG_HHO_SOURCE_ONE ? 1 : p->source == FHG_HHO_SOURCE_RANDOM_MODES ? 2 : 0};
    if (prm.source == 2) {
        // Modes m_id uniform in {1..4}, amplitudes N(0, 1) (Box-Muller), from the seed.
        uint64_t st = p->seed * 0x9E3779B97F4A7C15ull + 0x5EED;
        for (int i = 0; i < 4; i++) {
            for (int d = 0; d < 3; d++) prm.mode[i][d] = 1 + (int)(splitmix64(st) % 4);
            const double u1 = std::max(uniform01(st), 1e-300), u2 = uniform01(st);
            prm.amp[i] = std::sqrt(-2.0 * std::log(u1)) * std::cos(2 * kPi * u2);
        }
    }
    Rules rules;
    H->prm = prm;
    H->threads = threads;
    // cell: exact to degree 2k+2 (mass of P_{k+1}); face: degree 2k+1; RHS: high order.
    const int dim = p->dim;
    rules.cell = simplex_rule(dim, (2 * p->k + 2 + dim + 1) / 2 + 1);
    rules.cell_rhs = simplex_rule(dim, 6);
    rules.face = simplex_rule(dim - 1, (2 * p->k + 2 + dim) / 2 + 1);
    // Level hierarchy: standard coarsening while the system is above max_coarse_rows
    // (Multigrid::CoarseLevelNeeded, src/Solver/Multigrid/Multigrid.h:419-427) and n is even.
    int n = p->n;
    std::vector<int> ns;
    ns.push_back(n);
    const int nf = dim == 2 ? p->k + 1 : (p->k + 1) * (p->k + 2) / 2;
    H->block_size = nf;
    auto rows_of = [&](int m) -> long long {
        const long long faces = dim == 2 ? (long long)3 * m * m + 2 * m : (long long)12 * m * m * m + 6 * m * m;
        const long long bfaces = dim == 2 ? 4LL * m : 12LL * m * m;
        return (faces - bfaces) * nf;
    };
    while (true) {
        const int cur = ns.back();
        if (p->max_levels > 0 && (int)ns.size() >= p->max_levels) break;
        if (p->max_levels <= 0 && rows_of(cur) <= p->max_coarse_rows) break;
        if (cur % 2 != 0 || cur / 2 < 1) break;
        if (rows_of(cur / 2) == 0) break;
        ns.push_back(cur / 2);
    }
    H->levels.resize(ns.size());
    for (size_t l = 0; l < ns.size(); l++) {
        H->levels[l].mesh = dim == 2 ? build_tri(ns[l]) : build_tet(ns[l]);
        set_coefficients(H->levels[l].mesh, *p);
    }
    for (size_t l = 0; l + 1 < ns.size(); l++) link_coarse(H->levels[l].mesh, H->levels[l + 1].mesh);
    for (size_t l = 0; l < ns.size(); l++) {
        Level& L = H->levels[l];
        if (int rc = element_classes(L, prm, rules, threads, l == 0)) {
            H->err = "singular local HHO system";
            return rc;
        }
        assemble(L, prm, threads, l == 0);
        {   // the local operators by class, for condensing this level elsewhere (fhg_hho_level_tables)
            const ElementOps& O0 = L.cls_ops[0];
            L.cls_nC = O0.nC;
            L.cls_nFF = O0.nF * O0.nf;
            const size_t nH = (size_t)L.cls_nC + L.cls_nFF;
            L.cls_local.assign(L.cls_ops.size() * nH * nH, 0.0);
            for (size_t c = 0; c < L.cls_ops.size(); c++)
                if (L.cls_ops[c].local.a.size() == nH * nH)
                    std::copy(L.cls_ops[c].local.a.begin(), L.cls_ops[c].local.a.end(), L.cls_local.begin() + c * nH * nH);
        }
        if (l > 0) prolongation(H->levels[l - 1], L, prm, rules, threads, p->p_tables != 0);
        if (l > 1) {
            // element data of levels above the finest no longer needed (the finest keeps it for
            // the L2 error of a solution)
            std::vector<ElementOps>().swap(H->levels[l - 1].cls_ops);
        }
    }
    if (ns.size() > 1) std::vector<ElementOps>().swap(H->levels.back().cls_ops);
    H->rules = rules;
    return 0;
}

void fhg_hho_destroy(fhg_hho* h) { delete h; }

const char* fhg_hho_last_error(const fhg_hho* h) { return h ? h->err.c_str() : "null handle"; }

int fhg_hho_num_levels(const fhg_hho* h) { return h ? (int)h->levels.size() : 0; }

int fhg_hho_block_size(const fhg_hho* h) { return h ? h->block_size : 0; }

int fhg_hho_level(const fhg_hho* h, int l, int* n_rows, long long* nnz, const int** rowptr, const int** colidx,
                  const double** vals)
{
    if (!h || l < 0 || l >= (int)h->levels.size()) return -1;
    const Level& L = h->levels[l];
    if (n_rows) *n_rows = L.n_rows;
    if (nnz) *nnz = (long long)L.A_colidx.size();
    if (rowptr) *rowptr = L.A_rowptr.data();
    if (colidx) *colidx = L.A_colidx.data();
    if (vals) *vals = L.A_vals.data();
    return 0;
}

int fhg_hho_prolongation_table_sizes(const fhg_hho* h, int l, int* n_face_blocks, int* n_slots, int* n_coarse_elements,
                                     int* block_size, int* faces_per_element)
{
    if (!h || l < 0 || l + 1 >= (int)h->levels.size()) return -1;
    const Level& F = h->levels[l];
    if (F.Pt_ce.empty()) return -2;
    if (n_face_blocks) *n_face_blocks = F.mesh.n_interior;
    if (n_slots) *n_slots = F.Pt_nslots;
    if (n_coarse_elements) *n_coarse_elements = (int)h->levels[l + 1].mesh.el.size();
    if (block_size) *block_size = h->block_size;
    if (faces_per_element) *faces_per_element = F.mesh.dim + 1;
    return 0;
}

int fhg_hho_prolongation_tables(const fhg_hho* h, int l, int* face_ce, double* face_w, int* face_slot,
                                double* slot_contrib, int* coarse_elem_faces)
{
    if (!h || l < 0 || l + 1 >= (int)h->levels.size()) return -1;
    const Level& F = h->levels[l];
    if (F.Pt_ce.empty()) return -2;
    if (face_ce) std::copy(F.Pt_ce.begin(), F.Pt_ce.end(), face_ce);
    if (face_w) std::copy(F.Pt_w.begin(), F.Pt_w.end(), face_w);
    if (face_slot) std::copy(F.Pt_slot.begin(), F.Pt_slot.end(), face_slot);
    if (slot_contrib) std::copy(F.Pt_contrib.begin(), F.Pt_contrib.end(), slot_contrib);
    if (coarse_elem_faces) {
        const Mesh& MC = h->levels[l + 1].mesh;
        const int nF = MC.dim + 1;
        for (size_t e = 0; e < MC.el.size(); e++)
            for (int lf = 0; lf < nF; lf++) coarse_elem_faces[e * nF + lf] = MC.number[MC.ef[e][lf]];
    }
    return 0;
}

int fhg_hho_prolongation(const fhg_hho* h, int l, int* n_rows, int* n_cols, long long* nnz, const int** rowptr,
                         const int** colidx, const double** vals)
{
    if (!h || l < 0 || l + 1 >= (int)h->levels.size()) return -1;
    const Level& L = h->levels[l];
    if (n_rows) *n_rows = L.n_rows;
    if (n_cols) *n_cols = L.P_cols;
    if (nnz) *nnz = (long long)L.P_colidx.size();
    if (rowptr) *rowptr = L.P_rowptr.data();
    if (colidx) *colidx = L.P_colidx.data();
    if (vals) *vals = L.P_vals.data();
    return 0;
}

// Relative L2 error of the k+1 reconstruction of a face solution against the exact solution
// u = prod sin(pi x_i) of the sine source: cell unknowns recovered element by element
// (Diffusion_HHO::HybridCoeffsBySolvingCellUnknowns, src/Discretizations/HHO/Diffusion_HHO.h:855-882),
// reconstruction P [x_T; x_F] (ReconstructHigherOrderApproximationFromHybridCoeffs, :896-912), error
// sqrt(sum_T |u_h - u|^2_T) / sqrt(sum_T |u|^2_T) (Diffusion_HHO::L2Error, :120-150).
int fhg_hho_l2_error(const fhg_hho* h, const double* x, double* rel_error)
{
    if (!h || !x || !rel_error || h->levels.empty()) return -1;
    if (h->prm.source != 0) return -2;  // no closed-form solution for this source
    const Level& L = h->levels[0];
    const Mesh& M = L.mesh;
    const int dim = M.dim, nF = dim + 1, nf = h->block_size;
    const size_t ne = M.el.size();
    const int nthreads = std::max(1, h->threads);
    const size_t chunk = (ne + nthreads - 1) / nthreads;
    std::vector<double> err(nthreads, 0.0), nrm(nthreads, 0.0);
    std::vector<std::thread> th;
    for (int t = 0; t < nthreads; t++)
        th.emplace_back([&, t]() {
            const size_t e0 = t * chunk, e1 = std::min(ne, e0 + chunk);
            for (size_t e = e0; e < e1; e++) {
                const ElementOps& O = L.cls_ops[L.cls[e]];
                const auto xc = centroid(M, (int)e);
                const int nC = O.nC, nR = O.nR, nFF = nF * nf;
                std::vector<double> hyb(nC + nFF, 0.0);
                for (int lf = 0; lf < nF; lf++) {
                    const int g = M.number[M.ef[e][lf]];
                    if (g < 0) continue;
                    for (int a = 0; a < nf; a++) hyb[nC + lf * nf + a] = x[(size_t)g * nf + a];
                }
                for (int c = 0; c < nC; c++) {
                    double v = L.cell_rhs_e[e * nC + c];
                    for (int j = 0; j < nFF; j++) v += O.solve_cells(c, j) * hyb[nC + j];
                    hyb[c] = v;
                }
                std::vector<double> coef(nR, 0.0);
                for (int i = 0; i < nR; i++)
                    for (int j = 0; j < nC + nFF; j++) coef[i] += O.P(i, j) * hyb[j];
                const QPts Q = element_points(M, (int)e, h->rules.cell_rhs);
                double vals[64];
                for (size_t q = 0; q < Q.w.size(); q++) {
                    O.basis.eval_at(Q.x[q].data(), xc.data(), vals, nullptr);
                    double uh = 0;
                    for (int i = 0; i < nR; i++) uh += coef[i] * vals[i];
                    double u = 1.0;
                    for (int d = 0; d < dim; d++) u *= std::sin(kPi * Q.x[q][d]);
                    err[t] += Q.w[q] * (uh - u) * (uh - u);
                    nrm[t] += Q.w[q] * u * u;
                }
            }
        });
    for (auto& t : th) t.join();
    double E = 0, U = 0;
    for (int t = 0; t < nthreads; t++) { E += err[t]; U += nrm[t]; }
    *rel_error = U > 0 ? std::sqrt(E) / std::sqrt(U) : std::sqrt(E);
    return 0;
}

// Sizes of the post-processing tables of the finest level (fhg_hho_post_tables).
int fhg_hho_post_sizes(const fhg_hho* h, int* n_elements, int* n_classes, int* n_cell, int* n_face_dofs,
                       int* n_recon, int* n_points)
{
    if (!h || h->levels.empty()) return -1;
    const Level& L = h->levels[0];
    const ElementOps& O = L.cls_ops[0];
    if (n_elements) *n_elements = (int)L.mesh.el.size();
    if (n_classes) *n_classes = (int)L.cls_ops.size();
    if (n_cell) *n_cell = O.nC;
    if (n_face_dofs) *n_face_dofs = O.nF * O.nf;
    if (n_recon) *n_recon = O.nR;
    if (n_points) *n_points = (int)h->rules.cell_rhs.w.size();
    return 0;
}

// The finest level's data for recovering cell unknowns and evaluating the k+1 reconstruction
// (Diffusion_HHO.h:855-912) element by element: per element its class, the unknown block of each
// local face (-1: Dirichlet), its centroid (3 doubles) and A_TT^{-1} b_T; per class -A_TT^{-1} A_TF
// (nC x nFF), the reconstruction [nR x (nC + nFF)], and at the cell quadrature points (the rule of
// the L2 error) the weights, the offsets from the centroid (3 doubles each) and the reconstruction
// basis values (nq x nR). Elements of one class differ by a translation, so the offsets, weights and
// basis values of its first element serve them all.
int fhg_hho_post_tables(const fhg_hho* h, int* elem_class, int* elem_faces, double* elem_centre, double* cell_rhs,
                        double* solve_cells, double* recon, double* weights, double* offsets, double* basis)
{
    if (!h || h->levels.empty()) return -1;
    const Level& L = h->levels[0];
    const Mesh& M = L.mesh;
    const int dim = M.dim, nF = dim + 1;
    const size_t ne = M.el.size();
    const size_t ncls = L.cls_ops.size();
    const int nC = L.cls_ops[0].nC, nFF = nF * L.cls_ops[0].nf, nR = L.cls_ops[0].nR;
    const size_t nq = h->rules.cell_rhs.w.size();
    std::vector<long long> first(ncls, -1);
    for (size_t e = 0; e < ne; e++) {
        const int c = L.cls[e];
        if (first[c] < 0) first[c] = (long long)e;
        if (elem_class) elem_class[e] = c;
        if (elem_faces)
            for (int lf = 0; lf < nF; lf++) elem_faces[e * nF + lf] = M.number[M.ef[e][lf]];
        if (elem_centre) {
            const auto xc = centroid(M, (int)e);
            for (int d = 0; d < 3; d++) elem_centre[e * 3 + d] = xc[d];
        }
        if (cell_rhs)
            for (int c2 = 0; c2 < nC; c2++) cell_rhs[e * nC + c2] = L.cell_rhs_e[e * nC + c2];
    }
    for (size_t c = 0; c < ncls; c++) {
        const ElementOps& O = L.cls_ops[c];
        if (solve_cells)
            for (int i = 0; i < nC; i++)
                for (int j = 0; j < nFF; j++) solve_cells[(c * nC + i) * nFF + j] = O.solve_cells(i, j);
        if (recon)
            for (int i = 0; i < nR; i++)
                for (int j = 0; j < nC + nFF; j++) recon[(c * nR + i) * (nC + nFF) + j] = O.P(i, j);
        const int e = (int)first[c];
        if (e < 0) continue;
        const auto xc = centroid(M, e);
        const QPts Q = element_points(M, e, h->rules.cell_rhs);
        double vals[64];
        for (size_t q = 0; q < nq; q++) {
            if (weights) weights[c * nq + q] = Q.w[q];
            if (offsets)
                for (int d = 0; d < 3; d++) offsets[(c * nq + q) * 3 + d] = Q.x[q][d] - xc[d];
            if (basis) {
                O.basis.eval_at(Q.x[q].data(), xc.data(), vals, nullptr);
                for (int i = 0; i < nR; i++) basis[(c * nq + q) * nR + i] = vals[i];
            }
        }
    }
    return 0;
}

// The finest level's inputs of static condensation (Diffusion_HHO.h:627-638): per class the local
// operator before condensation, (nC + nFF)^2 row-major with the cell unknowns first; per element
// b_T = (f, c_j)_T; and for every unknown face block I its two elements with the face's local index
// in each, (e1, lf1, e2, lf2), in the order the assembly adds them.
int fhg_hho_condense_tables(const fhg_hho* h, double* local, double* b_cell, int* face_elems)
{
    if (!h || h->levels.empty()) return -1;
    const Level& L = h->levels[0];
    const Mesh& M = L.mesh;
    const int nF = M.dim + 1;
    const int nH = L.cls_ops[0].nC + nF * L.cls_ops[0].nf;
    if (local)
        for (size_t c = 0; c < L.cls_ops.size(); c++) {
            const Mat& A = L.cls_ops[c].local;
            if (A.a.size() != (size_t)nH * nH) return -3;
            for (int i = 0; i < nH; i++)
                for (int j = 0; j < nH; j++) local[(c * nH + i) * nH + j] = A(i, j);
        }
    if (b_cell) std::copy(L.bT_e.begin(), L.bT_e.end(), b_cell);
    if (face_elems)
        for (size_t f = 0; f < M.fv.size(); f++) {
            const int I = M.number[f];
            if (I < 0) continue;
            const int els[2] = {M.fe1[f], M.fe2[f]};
            for (int side = 0; side < 2; side++) {
                int lfi = -1;
                if (els[side] >= 0)
                    for (int lf = 0; lf < nF; lf++)
                        if (M.ef[els[side]][lf] == (int)f) lfi = lf;
                face_elems[(size_t)I * 4 + 2 * side] = els[side];
                face_elems[(size_t)I * 4 + 2 * side + 1] = lfi;
            }
        }
    return 0;
}

// Static-condensation inputs of level `level` (every level is rediscretised on its own mesh):
// sizes, then per element its class and its faces' unknown blocks (-1: Dirichlet), per class the
// local operator before condensation, per unknown face block its two elements and local faces.
int fhg_hho_level_sizes(const fhg_hho* h, int level, int* n_elements, int* n_classes, int* n_cell, int* n_face_dofs,
                        int* n_face_blocks)
{
    if (!h || level < 0 || level >= (int)h->levels.size()) return -1;
    const Level& L = h->levels[level];
    const size_t nH = (size_t)L.cls_nC + L.cls_nFF;
    if (nH == 0) return -1;
    if (n_elements) *n_elements = (int)L.mesh.el.size();
    if (n_classes) *n_classes = (int)(L.cls_local.size() / (nH * nH));
    if (n_cell) *n_cell = L.cls_nC;
    if (n_face_dofs) *n_face_dofs = L.cls_nFF;
    if (n_face_blocks) *n_face_blocks = L.mesh.n_interior;
    return 0;
}

int fhg_hho_level_tables(const fhg_hho* h, int level, int* elem_class, int* elem_faces, double* local, int* face_elems)
{
    if (!h || level < 0 || level >= (int)h->levels.size()) return -1;
    const Level& L = h->levels[level];
    const Mesh& M = L.mesh;
    const int nF = M.dim + 1;
    for (size_t e = 0; e < M.el.size(); e++) {
        if (elem_class) elem_class[e] = L.cls[e];
        if (elem_faces)
            for (int lf = 0; lf < nF; lf++) elem_faces[e * nF + lf] = M.number[M.ef[e][lf]];
    }
    if (local) std::copy(L.cls_local.begin(), L.cls_local.end(), local);
    if (face_elems)
        for (size_t f = 0; f < M.fv.size(); f++) {
            const int I = M.number[f];
            if (I < 0) continue;
            const int els[2] = {M.fe1[f], M.fe2[f]};
            for (int side = 0; side < 2; side++) {
                int lfi = -1;
                if (els[side] >= 0)
                    for (int lf = 0; lf < nF; lf++)
                        if (M.ef[els[side]][lf] == (int)f) lfi = lf;
                face_elems[(size_t)I * 4 + 2 * side] = els[side];
                face_elems[(size_t)I * 4 + 2 * side + 1] = lfi;
            }
        }
    return 0;
}

int fhg_hho_rhs(const fhg_hho* h, const double** b)
{
    if (!h || h->levels.empty()) return -1;
    *b = h->levels[0].b.data();
    return 0;
}

int fhg_hho_face_tensors(const fhg_hho* h, int l, double* out)
{
    if (!h || !out || l < 0 || l >= (int)h->levels.size()) return -1;
    const Mesh& M = h->levels[l].mesh;
    const int dim = M.dim;
    for (size_t f = 0; f < M.fv.size(); f++) {
        const int u = M.number[f];
        if (u < 0) continue;
        const int els[2] = {M.fe1[f], M.fe2[f]};
        for (int side = 0; side < 2; side++) {
            double* t = out + (size_t)u * 12 + side * 6;
            const auto& K = M.K[els[side]];
            if (dim == 3) {
                t[0] = K[0]; t[1] = K[4]; t[2] = K[8]; t[3] = K[1]; t[4] = K[2]; t[5] = K[5];
            } else {
                t[0] = K[0]; t[1] = K[3]; t[2] = K[1]; t[3] = 0; t[4] = 0; t[5] = 0;
            }
        }
    }
    return 0;
}

}  // extern "C"
