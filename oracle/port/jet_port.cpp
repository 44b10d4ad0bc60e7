// Oracle port — TEST INFRASTRUCTURE ONLY.
//
// A CPU restatement (C++17 + OpenMP) of the Jet pressure projection and the
// FLIP/PIC particle<->grid transfers. It exists to check the CUDA product and
// to time a CPU baseline; the product never links it. Every routine cites the
// reference function it restates (paths relative to the Jet source tree).
// Parity is pinned against the reference itself: tests compare this library
// bit-for-bit with the reference compiled from its own sources
// (oracle/ref_harness.cpp) and with the committed golden fixtures.
//
// Rounding rules: this file must be compiled with -ffp-contract=off so that
// double expressions round exactly like the reference built the same way.
// Reductions keep the reference's serial order (FdmBlas3::dot is a serial
// triple loop, src/jet/fdm_linear_system3.cpp:49-65).

#include "../oracle_api.h"

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

constexpr double kEpsD = std::numeric_limits<double>::epsilon();
constexpr double kMinWeight = 0.01;  // grid_fractional_..._solver3.cpp:25

struct Size3 {
    long x, y, z;
    long count() const { return x * y * z; }
};

inline long lin(const Size3& s, long i, long j, long k) {
    return i + s.x * (j + s.y * k);
}

// ---------------------------------------------------------------------------
// Sampling: LinearArraySampler3<double,double>::operator()
// (include/jet/detail/array_samplers3-inl.h:115-149), getBarycentric
// (include/jet/detail/math_utils-inl.h:147-172), trilerp (:177-211).

template <typename T>
inline void barycentric(T x, long iHigh, long* i, T* f) {
    T s = std::floor(x);
    *i = static_cast<long>(s);
    if (iHigh == 0) {
        *i = 0;
        *f = 0;
    } else if (*i < 0) {
        *i = 0;
        *f = 0;
    } else if (*i > iHigh - 1) {
        *i = iHigh - 1;
        *f = 1;
    } else {
        *f = static_cast<T>(x - s);
    }
}

template <typename T>
inline T lerp1(T a, T b, T f) {
    return (1 - f) * a + f * b;
}

template <typename V, typename T>
inline T trilinear(const V* data, const Size3& s, T nx, T ny, T nz) {
    long i, j, k;
    T fx, fy, fz;
    barycentric<T>(nx, s.x - 1, &i, &fx);
    barycentric<T>(ny, s.y - 1, &j, &fy);
    barycentric<T>(nz, s.z - 1, &k, &fz);
    long ip1 = std::min(i + 1, s.x - 1);
    long jp1 = std::min(j + 1, s.y - 1);
    long kp1 = std::min(k + 1, s.z - 1);
    T f000 = data[lin(s, i, j, k)], f100 = data[lin(s, ip1, j, k)];
    T f010 = data[lin(s, i, jp1, k)], f110 = data[lin(s, ip1, jp1, k)];
    T f001 = data[lin(s, i, j, kp1)], f101 = data[lin(s, ip1, j, kp1)];
    T f011 = data[lin(s, i, jp1, kp1)], f111 = data[lin(s, ip1, jp1, kp1)];
    T b0 = lerp1(lerp1(f000, f100, fx), lerp1(f010, f110, fx), fy);
    T b1 = lerp1(lerp1(f001, f101, fx), lerp1(f011, f111, fx), fy);
    return lerp1(b0, b1, fz);
}

struct Field {
    const orc_field* f;
    double sample(double x, double y, double z) const {
        if (f->kind == 0) return f->value;
        Size3 s{f->res[0], f->res[1], f->res[2]};
        double nx = (x - f->origin[0]) / f->spacing[0];
        double ny = (y - f->origin[1]) / f->spacing[1];
        double nz = (z - f->origin[2]) / f->spacing[2];
        return trilinear<double, double>(f->data, s, nx, ny, nz);
    }
};

// ---------------------------------------------------------------------------
// Level-set helpers (include/jet/detail/level_set_utils-inl.h:23-147).

inline bool inside(double phi) { return phi < 0; }

inline double fracInsideSdf(double p0, double p1) {
    if (inside(p0) && inside(p1)) return 1;
    if (inside(p0) && !inside(p1)) return p0 / (p0 - p1);
    if (!inside(p0) && inside(p1)) return p1 / (p1 - p0);
    return 0;
}

inline void cycle4(double* a) {
    double t = a[0];
    a[0] = a[1];
    a[1] = a[2];
    a[2] = a[3];
    a[3] = t;
}

double fracInside(double bl, double br, double tl, double tr) {
    int n = (bl < 0) + (tl < 0) + (br < 0) + (tr < 0);
    double l[4] = {bl, br, tr, tl};
    if (n == 4) return 1;
    if (n == 3) {
        while (l[0] < 0) cycle4(l);
        double s0 = 1 - fracInsideSdf(l[0], l[3]);
        double s1 = 1 - fracInsideSdf(l[0], l[1]);
        return 1 - 0.5f * s0 * s1;
    }
    if (n == 2) {
        while (l[0] >= 0 || !(l[1] < 0 || l[2] < 0)) cycle4(l);
        if (l[1] < 0) {
            double sl = fracInsideSdf(l[0], l[3]);
            double sr = fracInsideSdf(l[1], l[2]);
            return 0.5f * (sl + sr);
        }
        double mid = 0.25f * (l[0] + l[1] + l[2] + l[3]);
        if (mid < 0) {
            double area = 0;
            double s1 = 1 - fracInsideSdf(l[0], l[3]);
            double s3 = 1 - fracInsideSdf(l[2], l[3]);
            area += 0.5f * s1 * s3;
            double s2 = 1 - fracInsideSdf(l[2], l[1]);
            double s0 = 1 - fracInsideSdf(l[0], l[1]);
            area += 0.5f * s0 * s2;
            return 1 - area;
        }
        double area = 0;
        double s0 = fracInsideSdf(l[0], l[1]);
        double s1 = fracInsideSdf(l[0], l[3]);
        area += 0.5f * s0 * s1;
        double s2 = fracInsideSdf(l[2], l[1]);
        double s3 = fracInsideSdf(l[2], l[3]);
        area += 0.5f * s2 * s3;
        return area;
    }
    if (n == 1) {
        while (l[0] >= 0) cycle4(l);
        double s0 = fracInsideSdf(l[0], l[3]);
        double s1 = fracInsideSdf(l[0], l[1]);
        return 0.5f * s0 * s1;
    }
    return 0;
}

// ---------------------------------------------------------------------------
// FDM containers and BLAS (src/jet/fdm_linear_system3.cpp:37-134).

struct Row {
    double center, right, up, front;
};

struct Level {
    Size3 size;
    std::vector<Row> A;
    std::vector<double> x, b;
};

inline double offSum(const Row* A, const double* x, const Size3& s, long i,
                     long j, long k) {
    long c = lin(s, i, j, k);
    return ((i > 0) ? A[c - 1].right * x[c - 1] : 0.0) +
           ((i + 1 < s.x) ? A[c].right * x[c + 1] : 0.0) +
           ((j > 0) ? A[c - s.x].up * x[c - s.x] : 0.0) +
           ((j + 1 < s.y) ? A[c].up * x[c + s.x] : 0.0) +
           ((k > 0) ? A[c - s.x * s.y].front * x[c - s.x * s.y] : 0.0) +
           ((k + 1 < s.z) ? A[c].front * x[c + s.x * s.y] : 0.0);
}

// FdmBlas3::mvm (:79-96)
void mvm(const Row* A, const double* v, double* out, const Size3& s) {
#pragma omp parallel for schedule(static)
    for (long k = 0; k < s.z; ++k)
        for (long j = 0; j < s.y; ++j)
            for (long i = 0; i < s.x; ++i) {
                long c = lin(s, i, j, k);
                out[c] = A[c].center * v[c] +
                         ((i > 0) ? A[c - 1].right * v[c - 1] : 0.0) +
                         ((i + 1 < s.x) ? A[c].right * v[c + 1] : 0.0) +
                         ((j > 0) ? A[c - s.x].up * v[c - s.x] : 0.0) +
                         ((j + 1 < s.y) ? A[c].up * v[c + s.x] : 0.0) +
                         ((k > 0) ? A[c - s.x * s.y].front * v[c - s.x * s.y]
                                  : 0.0) +
                         ((k + 1 < s.z) ? A[c].front * v[c + s.x * s.y] : 0.0);
            }
}

// FdmBlas3::residual (:98-116)
void residual(const Row* A, const double* x, const double* b, double* r,
              const Size3& s) {
#pragma omp parallel for schedule(static)
    for (long k = 0; k < s.z; ++k)
        for (long j = 0; j < s.y; ++j)
            for (long i = 0; i < s.x; ++i) {
                long c = lin(s, i, j, k);
                r[c] = b[c] - A[c].center * x[c] -
                       ((i > 0) ? A[c - 1].right * x[c - 1] : 0.0) -
                       ((i + 1 < s.x) ? A[c].right * x[c + 1] : 0.0) -
                       ((j > 0) ? A[c - s.x].up * x[c - s.x] : 0.0) -
                       ((j + 1 < s.y) ? A[c].up * x[c + s.x] : 0.0) -
                       ((k > 0) ? A[c - s.x * s.y].front * x[c - s.x * s.y]
                                : 0.0) -
                       ((k + 1 < s.z) ? A[c].front * x[c + s.x * s.y] : 0.0);
            }
}

// FdmBlas3::dot (:49-65): serial, in index order.
double dot(const double* a, const double* b, long n) {
    double r = 0.0;
    for (long c = 0; c < n; ++c) r += a[c] * b[c];
    return r;
}

// FdmBlas3::axpy (:67-77): result = a*x + y.
void axpy(double a, const double* x, const double* y, double* out, long n) {
#pragma omp parallel for schedule(static)
    for (long c = 0; c < n; ++c) out[c] = a * x[c] + y[c];
}

// FdmGaussSeidelSolver3::relax (src/jet/fdm_gauss_seidel_solver3.cpp:103-120)
void relaxLex(const Row* A, const double* b, double w, double* x,
              const Size3& s) {
    for (long k = 0; k < s.z; ++k)
        for (long j = 0; j < s.y; ++j)
            for (long i = 0; i < s.x; ++i) {
                long c = lin(s, i, j, k);
                double r = offSum(A, x, s, i, j, k);
                x[c] = (1.0 - w) * x[c] + w * (b[c] - r) / A[c].center;
            }
}

// FdmGaussSeidelSolver3::relaxRedBlack (:150-221): red = (i+j+k) even first.
void relaxRB(const Row* A, const double* b, double w, double* x,
             const Size3& s) {
    for (int color = 0; color < 2; ++color) {
#pragma omp parallel for schedule(static)
        for (long k = 0; k < s.z; ++k)
            for (long j = 0; j < s.y; ++j)
                for (long i = (j + k + color) % 2; i < s.x; i += 2) {
                    long c = lin(s, i, j, k);
                    double r = offSum(A, x, s, i, j, k);
                    x[c] = (1.0 - w) * x[c] + w * (b[c] - r) / A[c].center;
                }
    }
}

// FdmMgUtils3::restrict (src/jet/fdm_mg_linear_system3.cpp:43-98)
void mgRestrict(const double* finer, double* coarser, const Size3& n) {
    static const double kern[4] = {0.125, 0.375, 0.375, 0.125};
    Size3 f{2 * n.x, 2 * n.y, 2 * n.z};
#pragma omp parallel for schedule(static)
    for (long k = 0; k < n.z; ++k) {
        long kI[4] = {(k > 0) ? 2 * k - 1 : 2 * k, 2 * k, 2 * k + 1,
                      (k + 1 < n.z) ? 2 * k + 2 : 2 * k + 1};
        for (long j = 0; j < n.y; ++j) {
            long jI[4] = {(j > 0) ? 2 * j - 1 : 2 * j, 2 * j, 2 * j + 1,
                          (j + 1 < n.y) ? 2 * j + 2 : 2 * j + 1};
            for (long i = 0; i < n.x; ++i) {
                long iI[4] = {(i > 0) ? 2 * i - 1 : 2 * i, 2 * i, 2 * i + 1,
                              (i + 1 < n.x) ? 2 * i + 2 : 2 * i + 1};
                double sum = 0.0;
                for (int z = 0; z < 4; ++z)
                    for (int y = 0; y < 4; ++y)
                        for (int x = 0; x < 4; ++x) {
                            double w = kern[x] * kern[y] * kern[z];
                            sum += w * finer[lin(f, iI[x], jI[y], kI[z])];
                        }
                coarser[lin(n, i, j, k)] = sum;
            }
        }
    }
}

// FdmMgUtils3::correct (:100-179). The k upper clamp compares with n.y, as
// the reference does (:159); identical for cubic grids.
void mgCorrect(const double* coarser, double* finer, const Size3& c) {
    Size3 n{2 * c.x, 2 * c.y, 2 * c.z};
#pragma omp parallel for schedule(static)
    for (long k = 0; k < n.z; ++k)
        for (long j = 0; j < n.y; ++j)
            for (long i = 0; i < n.x; ++i) {
                long ci = i / 2, cj = j / 2, ck = k / 2;
                long iI[2], jI[2], kI[2];
                double iW[2], jW[2], kW[2];
                if (i % 2 == 0) {
                    iI[0] = (i > 1) ? ci - 1 : ci; iI[1] = ci;
                    iW[0] = 0.25; iW[1] = 0.75;
                } else {
                    iI[0] = ci; iI[1] = (i + 1 < n.x) ? ci + 1 : ci;
                    iW[0] = 0.75; iW[1] = 0.25;
                }
                if (j % 2 == 0) {
                    jI[0] = (j > 1) ? cj - 1 : cj; jI[1] = cj;
                    jW[0] = 0.25; jW[1] = 0.75;
                } else {
                    jI[0] = cj; jI[1] = (j + 1 < n.y) ? cj + 1 : cj;
                    jW[0] = 0.75; jW[1] = 0.25;
                }
                if (k % 2 == 0) {
                    kI[0] = (k > 1) ? ck - 1 : ck; kI[1] = ck;
                    kW[0] = 0.25; kW[1] = 0.75;
                } else {
                    kI[0] = ck; kI[1] = (k + 1 < n.y) ? ck + 1 : ck;
                    kW[0] = 0.75; kW[1] = 0.25;
                }
                double& out = finer[lin(n, i, j, k)];
                for (int z = 0; z < 2; ++z)
                    for (int y = 0; y < 2; ++y)
                        for (int x = 0; x < 2; ++x) {
                            double w = iW[x] * jW[y] * kW[z] *
                                       coarser[lin(c, iI[x], jI[y], kI[z])];
                            out += w;
                        }
            }
}

// ---------------------------------------------------------------------------
// Multigrid-preconditioned CG (include/jet/detail/mg-inl.h:16-68,
// include/jet/detail/cg-inl.h:15-94, src/jet/fdm_mgpcg_solver3.cpp:15-80).

// Optional extra stop test, used only to state a CPU baseline at the same
// accuracy as the GPU solver: stop once ||b - A x||_2 <= g_rel_stop * ||b||_2
// (0 = the reference's own test only).
double g_rel_stop = 0.0;

struct MgSolver {
    orc_mg_params p;
    std::vector<Level>* levels;
    // Preconditioner work hierarchies (the reference copies three whole
    // hierarchies per call, fdm_mgpcg_solver3.cpp:24-26).
    std::vector<std::vector<double>> mx, mb, mbuf;

    void relax(int l, unsigned iters) {
        Level& L = (*levels)[l];
        for (unsigned it = 0; it < iters; ++it) {
            if (p.red_black)
                relaxRB(L.A.data(), mb[l].data(), p.sor, mx[l].data(), L.size);
            else
                relaxLex(L.A.data(), mb[l].data(), p.sor, mx[l].data(), L.size);
        }
    }

    void vcycle(int l) {
        Level& L = (*levels)[l];
        int nl = (int)levels->size();
        relax(l, p.restrict_iter);
        if (l < nl - 1) {
            residual(L.A.data(), mx[l].data(), mb[l].data(), mbuf[l].data(),
                     L.size);
            mgRestrict(mbuf[l].data(), mb[l + 1].data(), (*levels)[l + 1].size);
            std::fill(mx[l + 1].begin(), mx[l + 1].end(), 0.0);
            vcycle(l + 1);
            mgCorrect(mx[l + 1].data(), mx[l].data(), (*levels)[l + 1].size);
            relax(l, l > 0 ? p.correct_iter : p.final_iter);
        } else {
            relax(l, p.coarsest_iter);
            residual(L.A.data(), mx[l].data(), mb[l].data(), mbuf[l].data(),
                     L.size);
        }
        // The reference also evaluates a residual norm here whose value PCG
        // never reads (mg-inl.h:62-66); it does not change x.
        residual(L.A.data(), mx[l].data(), mb[l].data(), mbuf[l].data(),
                 L.size);
    }

    // Preconditioner::solve: x is both the initial guess and the output.
    void precond(const std::vector<double>& r, std::vector<double>& x) {
        size_t nl = levels->size();
        mx.resize(nl);
        mb.resize(nl);
        mbuf.resize(nl);
        for (size_t l = 0; l < nl; ++l) {
            // Copies of system->x: level 0 is overwritten below, coarse levels
            // hold the system's (zero) coarse x.
            mx[l] = (*levels)[l].x;
            mb[l] = (*levels)[l].x;
            mbuf[l] = (*levels)[l].x;
        }
        mx[0] = x;
        mb[0] = r;
        vcycle(0);
        x = mx[0];
    }

    bool solve(unsigned* iters_out, double* resid_out) {
        Level& F = (*levels)[0];
        long n = F.size.count();
        std::vector<double> r(n, 0.0), d(n, 0.0), q(n, 0.0), s(n, 0.0);
        std::fill(F.x.begin(), F.x.end(), 0.0);
        std::vector<double>& x = F.x;
        const std::vector<double>& b = F.b;

        residual(F.A.data(), x.data(), b.data(), r.data(), F.size);
        precond(r, d);
        double sigmaNew = dot(r.data(), d.data(), n);
        unsigned iter = 0;
        bool trigger = false;
        double tol = p.tolerance;
        const double bnorm = std::sqrt(dot(b.data(), b.data(), n));
        std::vector<double> tr;
        if (g_rel_stop > 0.0) tr.assign(n, 0.0);
        while (sigmaNew > tol * tol && iter < p.max_cg_iter) {
            mvm(F.A.data(), d.data(), q.data(), F.size);
            double alpha = sigmaNew / dot(d.data(), q.data(), n);
            axpy(alpha, d.data(), x.data(), x.data(), n);
            if (trigger || (iter % 50 == 0 && iter > 0)) {
                residual(F.A.data(), x.data(), b.data(), r.data(), F.size);
                trigger = false;
            } else {
                axpy(-alpha, q.data(), r.data(), r.data(), n);
            }
            precond(r, s);
            double sigmaOld = sigmaNew;
            sigmaNew = dot(r.data(), s.data(), n);
            if (sigmaNew > sigmaOld) trigger = true;
            double beta = sigmaNew / sigmaOld;
            axpy(beta, d.data(), s.data(), d.data(), n);
            ++iter;
            if (g_rel_stop > 0.0) {
                residual(F.A.data(), x.data(), b.data(), tr.data(), F.size);
                if (std::sqrt(dot(tr.data(), tr.data(), n)) <= g_rel_stop * bnorm)
                    break;
            }
        }
        *iters_out = iter;
        *resid_out = std::sqrt(std::fabs(sigmaNew));
        return *resid_out <= tol || iter < p.max_cg_iter;
    }
};

// FdmMgUtils3::resizeArrayWithFinest (detail/fdm_mg_linear_system3-inl.h:34-50)
std::vector<Size3> levelSizes(Size3 finest, unsigned maxLevels) {
    Size3 r = finest;
    unsigned i = 1;
    for (; i < maxLevels; ++i) {
        if (r.x % 2 == 0 && r.y % 2 == 0 && r.z % 2 == 0) {
            r.x >>= 1; r.y >>= 1; r.z >>= 1;
        } else {
            break;
        }
    }
    unsigned nl = std::max(i, 1u);
    std::vector<Size3> out(nl);
    Size3 c = r;
    for (unsigned l = 0; l < nl; ++l) {
        out[nl - l - 1] = c;
        c.x <<= 1; c.y <<= 1; c.z <<= 1;
    }
    return out;
}

// ---------------------------------------------------------------------------
// Fractional pressure solver (src/jet/grid_fractional_single_phase_pressure_solver3.cpp).

// Anonymous `restrict` for float pyramids (:29-115).
void restrictF(const std::vector<float>& finer, const Size3& fs,
               std::vector<float>& coarser, const Size3& n) {
    static const float centered[4] = {0.125f, 0.375f, 0.375f, 0.125f};
    static const float staggered[4] = {0.f, 1.f, 0.f, 0.f};
    int ks[3] = {fs.x != 2 * n.x ? 3 : 4, fs.y != 2 * n.y ? 3 : 4,
                 fs.z != 2 * n.z ? 3 : 4};
    const float* kx = ks[0] == 3 ? staggered : centered;
    const float* ky = ks[1] == 3 ? staggered : centered;
    const float* kz = ks[2] == 3 ? staggered : centered;
    auto idx = [](int ksz, long c, long nc, long out[4]) {
        if (ksz == 3) {
            out[0] = (c > 0) ? 2 * c - 1 : 2 * c;
            out[1] = 2 * c;
            out[2] = (c + 1 < nc) ? 2 * c + 1 : 2 * c;
            out[3] = 0;
        } else {
            out[0] = (c > 0) ? 2 * c - 1 : 2 * c;
            out[1] = 2 * c;
            out[2] = 2 * c + 1;
            out[3] = (c + 1 < nc) ? 2 * c + 2 : 2 * c + 1;
        }
    };
#pragma omp parallel for schedule(static)
    for (long k = 0; k < n.z; ++k) {
        long kI[4];
        idx(ks[2], k, n.z, kI);
        for (long j = 0; j < n.y; ++j) {
            long jI[4];
            idx(ks[1], j, n.y, jI);
            for (long i = 0; i < n.x; ++i) {
                long iI[4];
                idx(ks[0], i, n.x, iI);
                float sum = 0.0f;
                for (int z = 0; z < ks[2]; ++z)
                    for (int y = 0; y < ks[1]; ++y)
                        for (int x = 0; x < ks[0]; ++x) {
                            float w = kx[x] * ky[y] * kz[z];
                            sum += w * finer[lin(fs, iI[x], jI[y], kI[z])];
                        }
                coarser[lin(n, i, j, k)] = sum;
            }
        }
    }
}

struct PressureState {
    std::vector<Size3> sizes;
    std::vector<std::vector<float>> fluid, uw, vw, ww;
    std::vector<Level> levels;
};

PressureState g_state;

float faceWeight(double p0, double p1, double p2, double p3) {
    double frac = fracInside(p0, p1, p2, p3);
    double w = 1.0 - frac;
    w = (w < 0.0) ? 0.0 : ((w > 1.0) ? 1.0 : w);
    if (w < kMinWeight && w > 0.0) w = kMinWeight;
    return static_cast<float>(w);
}

// buildWeights (:520-636)
void buildWeights(const orc_grid* g, const orc_field* bsdf,
                  const orc_field* fsdf, unsigned maxLevels) {
    Size3 n{g->res[0], g->res[1], g->res[2]};
    PressureState& S = g_state;
    S.sizes = levelSizes(n, maxLevels);
    size_t nl = S.sizes.size();
    S.fluid.assign(nl, {});
    S.uw.assign(nl, {});
    S.vw.assign(nl, {});
    S.ww.assign(nl, {});
    for (size_t l = 0; l < nl; ++l) {
        Size3 s = S.sizes[l];
        S.fluid[l].assign(s.count(), 0.f);
        S.uw[l].assign((s.x + 1) * s.y * s.z, 0.f);
        S.vw[l].assign(s.x * (s.y + 1) * s.z, 0.f);
        S.ww[l].assign(s.x * s.y * (s.z + 1), 0.f);
    }
    const double hx = g->spacing[0], hy = g->spacing[1], hz = g->spacing[2];
    const double ox = g->origin[0], oy = g->origin[1], oz = g->origin[2];
    Field B{bsdf}, F{fsdf};
    // Face data origins (face_centered_grid3.cpp:440-442).
    const double uox = ox + 0.5 * 0.0, uoy = oy + 0.5 * hy, uoz = oz + 0.5 * hz;
    const double vox = ox + 0.5 * hx, voy = oy + 0.5 * 0.0, voz = oz + 0.5 * hz;
    const double wox = ox + 0.5 * hx, woy = oy + 0.5 * hy, woz = oz + 0.5 * 0.0;

#pragma omp parallel for schedule(static)
    for (long k = 0; k < n.z; ++k)
        for (long j = 0; j < n.y; ++j)
            for (long i = 0; i < n.x; ++i) {
                // Grid3::cellCenterPosition (grid3.cpp:32-38)
                double px = ox + hx * (i + 0.5);
                double py = oy + hy * (j + 0.5);
                double pz = oz + hz * (k + 0.5);
                S.fluid[0][lin(n, i, j, k)] =
                    static_cast<float>(F.sample(px, py, pz));
            }
    Size3 us{n.x + 1, n.y, n.z}, vs{n.x, n.y + 1, n.z}, ws{n.x, n.y, n.z + 1};
#pragma omp parallel for schedule(static)
    for (long k = 0; k < us.z; ++k)
        for (long j = 0; j < us.y; ++j)
            for (long i = 0; i < us.x; ++i) {
                double px = uox + hx * (double)i, py = uoy + hy * (double)j,
                       pz = uoz + hz * (double)k;
                double p0 = B.sample(px + 0.0, py + -0.5 * hy, pz + -0.5 * hz);
                double p1 = B.sample(px + 0.0, py + 0.5 * hy, pz + -0.5 * hz);
                double p2 = B.sample(px + 0.0, py + -0.5 * hy, pz + 0.5 * hz);
                double p3 = B.sample(px + 0.0, py + 0.5 * hy, pz + 0.5 * hz);
                S.uw[0][lin(us, i, j, k)] = faceWeight(p0, p1, p2, p3);
            }
#pragma omp parallel for schedule(static)
    for (long k = 0; k < vs.z; ++k)
        for (long j = 0; j < vs.y; ++j)
            for (long i = 0; i < vs.x; ++i) {
                double px = vox + hx * (double)i, py = voy + hy * (double)j,
                       pz = voz + hz * (double)k;
                double p0 = B.sample(px + -0.5 * hx, py + 0.0, pz + -0.5 * hz);
                double p1 = B.sample(px + -0.5 * hx, py + 0.0, pz + 0.5 * hz);
                double p2 = B.sample(px + 0.5 * hx, py + 0.0, pz + -0.5 * hz);
                double p3 = B.sample(px + 0.5 * hx, py + 0.0, pz + 0.5 * hz);
                S.vw[0][lin(vs, i, j, k)] = faceWeight(p0, p1, p2, p3);
            }
#pragma omp parallel for schedule(static)
    for (long k = 0; k < ws.z; ++k)
        for (long j = 0; j < ws.y; ++j)
            for (long i = 0; i < ws.x; ++i) {
                double px = wox + hx * (double)i, py = woy + hy * (double)j,
                       pz = woz + hz * (double)k;
                double p0 = B.sample(px + -0.5 * hx, py + -0.5 * hy, pz + 0.0);
                double p1 = B.sample(px + -0.5 * hx, py + 0.5 * hy, pz + 0.0);
                double p2 = B.sample(px + 0.5 * hx, py + -0.5 * hy, pz + 0.0);
                double p3 = B.sample(px + 0.5 * hx, py + 0.5 * hy, pz + 0.0);
                S.ww[0][lin(ws, i, j, k)] = faceWeight(p0, p1, p2, p3);
            }
    for (size_t l = 1; l < nl; ++l) {
        Size3 f = S.sizes[l - 1], c = S.sizes[l];
        restrictF(S.fluid[l - 1], f, S.fluid[l], c);
        restrictF(S.uw[l - 1], {f.x + 1, f.y, f.z}, S.uw[l], {c.x + 1, c.y, c.z});
        restrictF(S.vw[l - 1], {f.x, f.y + 1, f.z}, S.vw[l], {c.x, c.y + 1, c.z});
        restrictF(S.ww[l - 1], {f.x, f.y, f.z + 1}, S.ww[l], {c.x, c.y, c.z + 1});
    }
}

// buildSingleSystem (:117-267). u/v/w and solid velocities are only needed on
// the finest level (coarse right-hand sides are overwritten by restriction,
// include/jet/detail/mg-inl.h:28-30); they are NULL on coarse levels, where b
// is left at zero.
void buildSingleSystem(Level& L, const std::vector<float>& phi,
                       const std::vector<float>& uw,
                       const std::vector<float>& vw,
                       const std::vector<float>& ww, double hx, double hy,
                       double hz, const double* u, const double* v,
                       const double* w, const double* su, const double* sv,
                       const double* sw) {
    const Size3 n = L.size;
    Size3 us{n.x + 1, n.y, n.z}, vs{n.x, n.y + 1, n.z}, ws{n.x, n.y, n.z + 1};
    const double ihx = 1.0 / hx, ihy = 1.0 / hy, ihz = 1.0 / hz;
    const double ihx2 = ihx * ihx, ihy2 = ihy * ihy, ihz2 = ihz * ihz;
    L.A.assign(n.count(), Row{0, 0, 0, 0});
    L.b.assign(n.count(), 0.0);
    L.x.assign(n.count(), 0.0);
#pragma omp parallel for schedule(static)
    for (long k = 0; k < n.z; ++k)
        for (long j = 0; j < n.y; ++j)
            for (long i = 0; i < n.x; ++i) {
                long c = lin(n, i, j, k);
                Row& row = L.A[c];
                row.center = row.right = row.up = row.front = 0.0;
                double bb = 0.0;
                double cphi = phi[c];
                if (!inside(cphi)) {
                    row.center = 1.0;
                    L.b[c] = 0.0;
                    continue;
                }
                long uR = lin(us, i + 1, j, k), uL = lin(us, i, j, k);
                long vU = lin(vs, i, j + 1, k), vD = lin(vs, i, j, k);
                long wF = lin(ws, i, j, k + 1), wB = lin(ws, i, j, k);
                double term;
                if (i + 1 < n.x) {
                    term = uw[uR] * ihx2;
                    double nphi = phi[c + 1];
                    if (inside(nphi)) {
                        row.center += term;
                        row.right -= term;
                    } else {
                        double th = std::max(fracInsideSdf(cphi, nphi), 0.01);
                        row.center += term / th;
                    }
                    if (u) bb += uw[uR] * u[uR] * ihx;
                } else {
                    if (u) bb += u[uR] * ihx;
                }
                if (i > 0) {
                    term = uw[uL] * ihx2;
                    double nphi = phi[c - 1];
                    if (inside(nphi)) {
                        row.center += term;
                    } else {
                        double th = std::max(fracInsideSdf(cphi, nphi), 0.01);
                        row.center += term / th;
                    }
                    if (u) bb -= uw[uL] * u[uL] * ihx;
                } else {
                    if (u) bb -= u[uL] * ihx;
                }
                if (j + 1 < n.y) {
                    term = vw[vU] * ihy2;
                    double nphi = phi[c + n.x];
                    if (inside(nphi)) {
                        row.center += term;
                        row.up -= term;
                    } else {
                        double th = std::max(fracInsideSdf(cphi, nphi), 0.01);
                        row.center += term / th;
                    }
                    if (u) bb += vw[vU] * v[vU] * ihy;
                } else {
                    if (u) bb += v[vU] * ihy;
                }
                if (j > 0) {
                    term = vw[vD] * ihy2;
                    double nphi = phi[c - n.x];
                    if (inside(nphi)) {
                        row.center += term;
                    } else {
                        double th = std::max(fracInsideSdf(cphi, nphi), 0.01);
                        row.center += term / th;
                    }
                    if (u) bb -= vw[vD] * v[vD] * ihy;
                } else {
                    if (u) bb -= v[vD] * ihy;
                }
                if (k + 1 < n.z) {
                    term = ww[wF] * ihz2;
                    double nphi = phi[c + n.x * n.y];
                    if (inside(nphi)) {
                        row.center += term;
                        row.front -= term;
                    } else {
                        double th = std::max(fracInsideSdf(cphi, nphi), 0.01);
                        row.center += term / th;
                    }
                    if (u) bb += ww[wF] * w[wF] * ihz;
                } else {
                    if (u) bb += w[wF] * ihz;
                }
                if (k > 0) {
                    term = ww[wB] * ihz2;
                    double nphi = phi[c - n.x * n.y];
                    if (inside(nphi)) {
                        row.center += term;
                    } else {
                        double th = std::max(fracInsideSdf(cphi, nphi), 0.01);
                        row.center += term / th;
                    }
                    if (u) bb -= ww[wB] * w[wB] * ihz;
                } else {
                    if (u) bb -= w[wB] * ihz;
                }
                if (u) {
                    double sR = su ? su[uR] : 0.0, sL = su ? su[uL] : 0.0;
                    double sU = sv ? sv[vU] : 0.0, sD = sv ? sv[vD] : 0.0;
                    double sF = sw ? sw[wF] : 0.0, sB = sw ? sw[wB] : 0.0;
                    double contrib = (1.0 - uw[uR]) * sR * ihx -
                                     (1.0 - uw[uL]) * sL * ihx +
                                     (1.0 - vw[vU]) * sU * ihy -
                                     (1.0 - vw[vD]) * sD * ihy +
                                     (1.0 - ww[wF]) * sF * ihz -
                                     (1.0 - ww[wB]) * sB * ihz;
                    bb += contrib;
                }
                if (row.center < kEpsD) {
                    row.center = 1.0;
                    bb = 0.0;
                }
                L.b[c] = bb;
            }
}

// applyPressureGradient (:715-765). out_* start as copies of the input.
void applyGradient(const orc_grid* g, const double* x, const double* u,
                   const double* v, const double* w, double* ou, double* ov,
                   double* ow) {
    const PressureState& S = g_state;
    Size3 n{g->res[0], g->res[1], g->res[2]};
    Size3 us{n.x + 1, n.y, n.z}, vs{n.x, n.y + 1, n.z}, ws{n.x, n.y, n.z + 1};
    const double ihx = 1.0 / g->spacing[0], ihy = 1.0 / g->spacing[1],
                 ihz = 1.0 / g->spacing[2];
    const std::vector<float>& phi = S.fluid[0];
#pragma omp parallel for schedule(static)
    for (long k = 0; k < n.z; ++k)
        for (long j = 0; j < n.y; ++j)
            for (long i = 0; i < n.x; ++i) {
                long c = lin(n, i, j, k);
                double cphi = phi[c];
                if (i + 1 < n.x && S.uw[0][lin(us, i + 1, j, k)] > 0.0 &&
                    (inside(cphi) || inside(phi[c + 1]))) {
                    double th = std::max(fracInsideSdf(cphi, phi[c + 1]), 0.01);
                    long f = lin(us, i + 1, j, k);
                    ou[f] = u[f] + ihx / th * (x[c + 1] - x[c]);
                }
                if (j + 1 < n.y && S.vw[0][lin(vs, i, j + 1, k)] > 0.0 &&
                    (inside(cphi) || inside(phi[c + n.x]))) {
                    double th =
                        std::max(fracInsideSdf(cphi, phi[c + n.x]), 0.01);
                    long f = lin(vs, i, j + 1, k);
                    ov[f] = v[f] + ihy / th * (x[c + n.x] - x[c]);
                }
                if (k + 1 < n.z && S.ww[0][lin(ws, i, j, k + 1)] > 0.0 &&
                    (inside(cphi) || inside(phi[c + n.x * n.y]))) {
                    double th = std::max(
                        fracInsideSdf(cphi, phi[c + n.x * n.y]), 0.01);
                    long f = lin(ws, i, j, k + 1);
                    ow[f] = w[f] + ihz / th * (x[c + n.x * n.y] - x[c]);
                }
            }
}

// LinearArraySampler3::getCoordinatesAndWeights (array_samplers3-inl.h:151-193)
struct Stencil {
    long idx[8];
    double w[8];
};

inline void coordsAndWeights(const Size3& s, double ox, double oy, double oz,
                             double ihx, double ihy, double ihz, double px,
                             double py, double pz, Stencil* st) {
    double nx = (px - ox) * ihx, ny = (py - oy) * ihy, nz = (pz - oz) * ihz;
    long i, j, k;
    double fx, fy, fz;
    barycentric<double>(nx, s.x - 1, &i, &fx);
    barycentric<double>(ny, s.y - 1, &j, &fy);
    barycentric<double>(nz, s.z - 1, &k, &fz);
    long ip1 = std::min(i + 1, s.x - 1);
    long jp1 = std::min(j + 1, s.y - 1);
    long kp1 = std::min(k + 1, s.z - 1);
    st->idx[0] = lin(s, i, j, k);
    st->idx[1] = lin(s, ip1, j, k);
    st->idx[2] = lin(s, i, jp1, k);
    st->idx[3] = lin(s, ip1, jp1, k);
    st->idx[4] = lin(s, i, j, kp1);
    st->idx[5] = lin(s, ip1, j, kp1);
    st->idx[6] = lin(s, i, jp1, kp1);
    st->idx[7] = lin(s, ip1, jp1, kp1);
    st->w[0] = (1 - fx) * (1 - fy) * (1 - fz);
    st->w[1] = fx * (1 - fy) * (1 - fz);
    st->w[2] = (1 - fx) * fy * (1 - fz);
    st->w[3] = fx * fy * (1 - fz);
    st->w[4] = (1 - fx) * (1 - fy) * fz;
    st->w[5] = fx * (1 - fy) * fz;
    st->w[6] = (1 - fx) * fy * fz;
    st->w[7] = fx * fy * fz;
}

struct FaceGeom {
    Size3 s;
    double o[3];
};

void faceGeoms(const orc_grid* g, FaceGeom fg[3]) {
    Size3 n{g->res[0], g->res[1], g->res[2]};
    const double* h = g->spacing;
    const double* o = g->origin;
    fg[0] = {{n.x + 1, n.y, n.z}, {o[0] + 0.5 * 0.0, o[1] + 0.5 * h[1], o[2] + 0.5 * h[2]}};
    fg[1] = {{n.x, n.y + 1, n.z}, {o[0] + 0.5 * h[0], o[1] + 0.5 * 0.0, o[2] + 0.5 * h[2]}};
    fg[2] = {{n.x, n.y, n.z + 1}, {o[0] + 0.5 * h[0], o[1] + 0.5 * h[1], o[2] + 0.5 * 0.0}};
}

int g_threads = 0;

}  // namespace

extern "C" {

void orc_set_relative_stop(double rel) { g_rel_stop = rel > 0.0 ? rel : 0.0; }

void orc_set_threads(int n) {
    g_threads = n;
#ifdef _OPENMP
    omp_set_num_threads(n > 0 ? n : omp_get_num_procs());
#endif
}

int orc_pressure_solve(const orc_grid* g, const double* u, const double* v,
                       const double* w, const orc_field* boundary_sdf,
                       const orc_field* fluid_sdf, const double* solid_u,
                       const double* solid_v, const double* solid_w,
                       const orc_mg_params* p, double* out_u, double* out_v,
                       double* out_w, double* out_p, unsigned int* iters,
                       double* resid) {
    PressureState& S = g_state;
    buildWeights(g, boundary_sdf, fluid_sdf, p->max_levels);
    size_t nl = S.sizes.size();
    S.levels.assign(nl, {});
    // buildSystem (:651-713): the finest level uses the input velocity; the
    // coarse levels' b is dead (see buildSingleSystem above).
    double hx = g->spacing[0], hy = g->spacing[1], hz = g->spacing[2];
    for (size_t l = 0; l < nl; ++l) {
        S.levels[l].size = S.sizes[l];
        if (l > 0) {
            hx *= 2.0;
            hy *= 2.0;
            hz *= 2.0;
        }
        buildSingleSystem(S.levels[l], S.fluid[l], S.uw[l], S.vw[l], S.ww[l],
                          hx, hy, hz, l == 0 ? u : nullptr,
                          l == 0 ? v : nullptr, l == 0 ? w : nullptr,
                          solid_u, solid_v, solid_w);
    }
    MgSolver solver{*p, &S.levels, {}, {}, {}};
    unsigned it = 0;
    double rs = 0;
    bool ok = solver.solve(&it, &rs);
    if (iters) *iters = it;
    if (resid) *resid = rs;
    Size3 n{g->res[0], g->res[1], g->res[2]};
    long nu = (n.x + 1) * n.y * n.z, nv = n.x * (n.y + 1) * n.z,
         nw = n.x * n.y * (n.z + 1);
    if (out_u != u) std::memcpy(out_u, u, nu * sizeof(double));
    if (out_v != v) std::memcpy(out_v, v, nv * sizeof(double));
    if (out_w != w) std::memcpy(out_w, w, nw * sizeof(double));
    // The reference reads the input grid while writing the output grid; when
    // they alias, read from a copy.
    std::vector<double> cu(u, u + nu), cv(v, v + nv), cw(w, w + nw);
    applyGradient(g, S.levels[0].x.data(), cu.data(), cv.data(), cw.data(),
                  out_u, out_v, out_w);
    if (out_p)
        std::memcpy(out_p, S.levels[0].x.data(), n.count() * sizeof(double));
    return ok ? 1 : 0;
}

int orc_level_count(void) { return (int)g_state.sizes.size(); }

long orc_get_level(int level, int what, void* dst, size_t capacity) {
    PressureState& S = g_state;
    if (level < 0 || level >= (int)S.sizes.size()) return -1;
    // Copies n elements of `size` bytes if they fit the caller's buffer.
    auto put = [&](const void* src, size_t n, size_t size) -> long {
        if (n * size > capacity) return -2;
        std::memcpy(dst, src, n * size);
        return (long)n;
    };
    switch (what) {
        case 0: return put(S.fluid[level].data(), S.fluid[level].size(), 4);
        case 1: return put(S.uw[level].data(), S.uw[level].size(), 4);
        case 2: return put(S.vw[level].data(), S.vw[level].size(), 4);
        case 3: return put(S.ww[level].data(), S.ww[level].size(), 4);
        case 4: {
            if (level >= (int)S.levels.size()) return -1;
            const Level& L = S.levels[level];
            return put(L.A.data(), L.A.size(), sizeof(Row));
        }
        case 5: {
            if (level >= (int)S.levels.size()) return -1;
            const Level& L = S.levels[level];
            return put(L.b.data(), L.b.size(), sizeof(double));
        }
        default:
            return -1;
    }
}

int orc_mgpcg_system(const int res0[3], int levels, const double* A,
                     const double* b, const orc_mg_params* p, double* x0,
                     unsigned int* iters, double* resid) {
    std::vector<Level> L(levels);
    long off = 0;
    for (int l = 0; l < levels; ++l) {
        Size3 s{res0[0] >> l, res0[1] >> l, res0[2] >> l};
        L[l].size = s;
        long n = s.count();
        L[l].A.resize(n);
        std::memcpy(L[l].A.data(), A + 4 * off, n * sizeof(Row));
        L[l].b.assign(b + off, b + off + n);
        L[l].x.assign(n, 0.0);
        off += n;
    }
    MgSolver solver{*p, &L, {}, {}, {}};
    unsigned it = 0;
    double rs = 0;
    bool ok = solver.solve(&it, &rs);
    if (iters) *iters = it;
    if (resid) *resid = rs;
    std::memcpy(x0, L[0].x.data(), L[0].x.size() * sizeof(double));
    return ok ? 1 : 0;
}

void orc_relax(const int res[3], const double* A, const double* b, double sor,
               int red_black, int sweeps, double* x) {
    Size3 s{res[0], res[1], res[2]};
    const Row* R = reinterpret_cast<const Row*>(A);
    for (int it = 0; it < sweeps; ++it) {
        if (red_black)
            relaxRB(R, b, sor, x, s);
        else
            relaxLex(R, b, sor, x, s);
    }
}

void orc_mg_restrict(const int coarse_res[3], const double* finer,
                     double* coarser) {
    mgRestrict(finer, coarser, {coarse_res[0], coarse_res[1], coarse_res[2]});
}

void orc_mg_correct(const int coarse_res[3], const double* coarser,
                    double* finer) {
    mgCorrect(coarser, finer, {coarse_res[0], coarse_res[1], coarse_res[2]});
}

void orc_residual(const int res[3], const double* A, const double* x,
                  const double* b, double* r) {
    residual(reinterpret_cast<const Row*>(A), x, b, r,
             {res[0], res[1], res[2]});
}

double orc_dot(long n, const double* a, const double* b) {
    return dot(a, b, n);
}

void orc_p2g(const orc_grid* g, long np, const double* pos, const double* vel,
             double* u, double* v, double* w, char* mu, char* mv, char* mw,
             float* snap_u, float* snap_v, float* snap_w) {
    FaceGeom fg[3];
    faceGeoms(g, fg);
    double* grids[3] = {u, v, w};
    char* marks[3] = {mu, mv, mw};
    float* snaps[3] = {snap_u, snap_v, snap_w};
    const double ih[3] = {1.0 / g->spacing[0], 1.0 / g->spacing[1],
                          1.0 / g->spacing[2]};
    std::vector<double> wsum[3];
    for (int a = 0; a < 3; ++a) {
        long n = fg[a].s.count();
        std::fill(grids[a], grids[a] + n, 0.0);
        wsum[a].assign(n, 0.0);
        if (marks[a]) std::fill(marks[a], marks[a] + n, 0);
    }
    // Serial scatter in particle order (pic_solver3.cpp:152-176).
    for (long p = 0; p < np; ++p) {
        for (int a = 0; a < 3; ++a) {
            Stencil st;
            coordsAndWeights(fg[a].s, fg[a].o[0], fg[a].o[1], fg[a].o[2], ih[0],
                             ih[1], ih[2], pos[3 * p], pos[3 * p + 1],
                             pos[3 * p + 2], &st);
            for (int q = 0; q < 8; ++q) {
                grids[a][st.idx[q]] += vel[3 * p + a] * st.w[q];
                wsum[a][st.idx[q]] += st.w[q];
                if (marks[a]) marks[a][st.idx[q]] = 1;
            }
        }
    }
    for (int a = 0; a < 3; ++a) {
        long n = fg[a].s.count();
#pragma omp parallel for schedule(static)
        for (long c = 0; c < n; ++c)
            if (wsum[a][c] > 0.0) grids[a][c] /= wsum[a][c];
        if (snaps[a])
            for (long c = 0; c < n; ++c)
                snaps[a][c] = static_cast<float>(grids[a][c]);
    }
}

void orc_g2p_flip(const orc_grid* g, long np, const double* pos, double* vel,
                  const double* u, const double* v, const double* w,
                  float* snap_u, float* snap_v, float* snap_w,
                  double pic_blend) {
    FaceGeom fg[3];
    faceGeoms(g, fg);
    const double* grids[3] = {u, v, w};
    float* snaps[3] = {snap_u, snap_v, snap_w};
    for (int a = 0; a < 3; ++a) {
        long n = fg[a].s.count();
#pragma omp parallel for schedule(static)
        for (long c = 0; c < n; ++c)
            snaps[a][c] = static_cast<float>(grids[a][c]) - snaps[a][c];
    }
    // LinearArraySampler3<float,float> over the deltas with float geometry
    // (flip_solver3.cpp:72-88).
    const float hf[3] = {(float)g->spacing[0], (float)g->spacing[1],
                         (float)g->spacing[2]};
    float of[3][3];
    for (int a = 0; a < 3; ++a)
        for (int d = 0; d < 3; ++d) of[a][d] = (float)fg[a].o[d];
    const double ih[3] = {1.0 / g->spacing[0], 1.0 / g->spacing[1],
                          1.0 / g->spacing[2]};
    (void)ih;
#pragma omp parallel for schedule(static)
    for (long p = 0; p < np; ++p) {
        float xf[3] = {(float)pos[3 * p], (float)pos[3 * p + 1],
                       (float)pos[3 * p + 2]};
        double flip[3];
        for (int a = 0; a < 3; ++a) {
            float nx = (xf[0] - of[a][0]) / hf[0];
            float ny = (xf[1] - of[a][1]) / hf[1];
            float nz = (xf[2] - of[a][2]) / hf[2];
            double d = (double)trilinear<float, float>(snaps[a], fg[a].s, nx,
                                                       ny, nz);
            flip[a] = vel[3 * p + a] + d;
        }
        if (pic_blend > 0.0) {
            double pic[3];
            for (int a = 0; a < 3; ++a) {
                double nx = (pos[3 * p] - fg[a].o[0]) / g->spacing[0];
                double ny = (pos[3 * p + 1] - fg[a].o[1]) / g->spacing[1];
                double nz = (pos[3 * p + 2] - fg[a].o[2]) / g->spacing[2];
                pic[a] = trilinear<double, double>(grids[a], fg[a].s, nx, ny,
                                                   nz);
            }
            for (int a = 0; a < 3; ++a)
                flip[a] = (1 - pic_blend) * flip[a] + pic_blend * pic[a];
        }
        for (int a = 0; a < 3; ++a) vel[3 * p + a] = flip[a];
    }
}

// GridFractionalBoundaryConditionSolver3::constrainVelocity
// (src/jet/grid_fractional_boundary_condition_solver3.cpp:26-233).
void orc_constrain_velocity(const orc_grid* g, double* u, double* v,
                            double* w, const orc_field* sdf,
                            const orc_collider* col, int closed,
                            unsigned int depth) {
    FaceGeom fg[3];
    faceGeoms(g, fg);
    const double* h = g->spacing;
    double* vel[3] = {u, v, w};
    Field F{sdf};
    // RigidBodyCollider3::velocityAt (rigid_body_collider3.cpp:25-28) and
    // Vector3::cross (include/jet/detail/vector3-inl.h:125-127).
    auto colVel = [&](const double p[3], double out[3]) {
        if (col == nullptr) {
            out[0] = out[1] = out[2] = 0.0;
            return;
        }
        const double* a = col->ang;
        const double r[3] = {p[0] - col->centre[0], p[1] - col->centre[1],
                             p[2] - col->centre[2]};
        const double cr[3] = {a[1] * r[2] - r[1] * a[2],
                              a[2] * r[0] - r[2] * a[0],
                              a[0] * r[1] - r[0] * a[1]};
        for (int d = 0; d < 3; ++d) out[d] = col->lin[d] + cr[d];
    };
    auto facePos = [&](int a, long i, long j, long k, double p[3]) {
        p[0] = fg[a].o[0] + h[0] * (double)i;
        p[1] = fg[a].o[1] + h[1] * (double)j;
        p[2] = fg[a].o[2] + h[2] * (double)k;
    };
    // Collider velocity and markers (:51-100).
    std::vector<char> marker[3];
    for (int a = 0; a < 3; ++a) {
        const Size3 s = fg[a].s;
        marker[a].assign(s.count(), 1);
#pragma omp parallel for schedule(static)
        for (long k = 0; k < s.z; ++k)
            for (long j = 0; j < s.y; ++j)
                for (long i = 0; i < s.x; ++i) {
                    double p[3], q0[3], q1[3];
                    facePos(a, i, j, k, p);
                    for (int d = 0; d < 3; ++d) {
                        const double off = d == a ? 0.5 * h[d] : 0.0;
                        q0[d] = p[d] - off;
                        q1[d] = p[d] + off;
                    }
                    double frac = fracInsideSdf(F.sample(q0[0], q0[1], q0[2]),
                                                F.sample(q1[0], q1[1], q1[2]));
                    frac = 1.0 - (frac < 0.0 ? 0.0 : frac > 1.0 ? 1.0 : frac);
                    const long c = lin(s, i, j, k);
                    if (frac > 0.0) {
                        marker[a][c] = 1;
                    } else {
                        double cv[3];
                        colVel(p, cv);
                        vel[a][c] = cv[a];
                        marker[a][c] = 0;
                    }
                }
    }
    // Free slip: extrapolate into the collider (:102-108).
    for (int a = 0; a < 3; ++a) {
        const int res[3] = {(int)fg[a].s.x, (int)fg[a].s.y, (int)fg[a].s.z};
        orc_extrapolate(res, vel[a], marker[a].data(), depth);
    }
    // ScalarGrid3::gradient (src/jet/scalar_grid3.cpp:89-102) over the
    // central differences of gradient3 (src/jet/fdm_utils.cpp:49-67).
    auto gradient = [&](const double p[3], double gout[3]) {
        gout[0] = gout[1] = gout[2] = 0.0;
        if (sdf == nullptr || sdf->kind == 0) return;
        const Size3 s{sdf->res[0], sdf->res[1], sdf->res[2]};
        Stencil st;
        coordsAndWeights(s, sdf->origin[0], sdf->origin[1], sdf->origin[2],
                         1.0 / sdf->spacing[0], 1.0 / sdf->spacing[1],
                         1.0 / sdf->spacing[2], p[0], p[1], p[2], &st);
        const double* d = sdf->data;
        for (int n = 0; n < 8; ++n) {
            const long c = st.idx[n];
            const long i = c % s.x, j = (c / s.x) % s.y, k = c / (s.x * s.y);
            const double l = d[lin(s, i > 0 ? i - 1 : i, j, k)];
            const double r = d[lin(s, i + 1 < s.x ? i + 1 : i, j, k)];
            const double dn = d[lin(s, i, j > 0 ? j - 1 : j, k)];
            const double up = d[lin(s, i, j + 1 < s.y ? j + 1 : j, k)];
            const double b = d[lin(s, i, j, k > 0 ? k - 1 : k)];
            const double f = d[lin(s, i, j, k + 1 < s.z ? k + 1 : k)];
            const double gv[3] = {0.5 * (r - l) / sdf->spacing[0],
                                  0.5 * (up - dn) / sdf->spacing[1],
                                  0.5 * (f - b) / sdf->spacing[2]};
            for (int q = 0; q < 3; ++q) gout[q] = gout[q] + st.w[n] * gv[q];
        }
    };
    // No flux: project onto the collider's tangent plane (:110-175), reading
    // the extrapolated field, writing temporaries.
    std::vector<double> tmp[3];
    for (int a = 0; a < 3; ++a) {
        const Size3 s = fg[a].s;
        tmp[a].resize(s.count());
#pragma omp parallel for schedule(static)
        for (long k = 0; k < s.z; ++k)
            for (long j = 0; j < s.y; ++j)
                for (long i = 0; i < s.x; ++i) {
                    const long c = lin(s, i, j, k);
                    double p[3];
                    facePos(a, i, j, k, p);
                    if (!inside(F.sample(p[0], p[1], p[2]))) {
                        tmp[a][c] = vel[a][c];
                        continue;
                    }
                    double cv[3], fv[3], gd[3];
                    colVel(p, cv);
                    for (int b = 0; b < 3; ++b) {  // FaceCenteredGrid3::sample
                        const double nx = (p[0] - fg[b].o[0]) / h[0];
                        const double ny = (p[1] - fg[b].o[1]) / h[1];
                        const double nz = (p[2] - fg[b].o[2]) / h[2];
                        fv[b] = trilinear<double, double>(vel[b], fg[b].s, nx,
                                                          ny, nz);
                    }
                    gradient(p, gd);
                    if (gd[0] * gd[0] + gd[1] * gd[1] + gd[2] * gd[2] > 0.0) {
                        const double len =
                            std::sqrt(gd[0] * gd[0] + gd[1] * gd[1] + gd[2] * gd[2]);
                        const double n[3] = {gd[0] / len, gd[1] / len, gd[2] / len};
                        const double vr[3] = {fv[0] - cv[0], fv[1] - cv[1],
                                              fv[2] - cv[2]};
                        // projectAndApplyFriction (src/jet/physics_helpers.h:34-45).
                        const double dn = vr[0] * n[0] + vr[1] * n[1] + vr[2] * n[2];
                        double vt[3] = {vr[0] - n[0] * dn, vr[1] - n[1] * dn,
                                        vr[2] - n[2] * dn};
                        const double l2 = vt[0] * vt[0] + vt[1] * vt[1] + vt[2] * vt[2];
                        if (l2 > 0) {
                            const double veln = std::max(-dn, 0.0);
                            const double fr = col ? col->friction : 0.0;
                            const double sc = std::max(
                                1.0 - fr * veln / std::sqrt(l2), 0.0);
                            for (int q = 0; q < 3; ++q) vt[q] = vt[q] * sc;
                        }
                        tmp[a][c] = vt[a] + cv[a];
                    } else {
                        tmp[a][c] = cv[a];
                    }
                }
    }
    // Transfer results, then zero the normal velocity on closed domain
    // faces (:177-232).
    for (int a = 0; a < 3; ++a) {
        std::memcpy(vel[a], tmp[a].data(), sizeof(double) * tmp[a].size());
        const Size3 s = fg[a].s;
        const int lo = 1 << (2 * a), hi = 1 << (2 * a + 1);
        const long ext[3] = {s.x, s.y, s.z};
        for (long k = 0; k < s.z; ++k)
            for (long j = 0; j < s.y; ++j)
                for (long i = 0; i < s.x; ++i) {
                    const long idx[3] = {i, j, k};
                    if (((closed & lo) && idx[a] == 0) ||
                        ((closed & hi) && idx[a] == ext[a] - 1))
                        vel[a][lin(s, i, j, k)] = 0.0;
                }
    }
}

// PicSolver3::moveParticles (src/jet/pic_solver3.cpp:206-282) and
// Collider3::resolveCollision (src/jet/collider3.cpp:19-73) with radius 0
// and restitution 0 against a transformed Sphere3 (src/jet/sphere3.cpp:25-39,
// src/jet/surface3.cpp:23-79, include/jet/detail/transform3-inl.h:45-79).
void orc_move_particles(const orc_grid* g, long np, double* pos, double* vel,
                        const double* u, const double* v, const double* w,
                        double dt, double max_cfl, int closed,
                        const orc_collider* col, const orc_sphere* sph) {
    FaceGeom fg[3];
    faceGeoms(g, fg);
    const double* grids[3] = {u, v, w};
    const double* h = g->spacing;
    auto sample = [&](const double p[3], double out[3]) {
        for (int a = 0; a < 3; ++a) {
            const double nx = (p[0] - fg[a].o[0]) / h[0];
            const double ny = (p[1] - fg[a].o[1]) / h[1];
            const double nz = (p[2] - fg[a].o[2]) / h[2];
            out[a] = trilinear<double, double>(grids[a], fg[a].s, nx, ny, nz);
        }
    };
    double lo[3], hi[3];  // Grid3::boundingBox (src/jet/grid3.cpp:77)
    for (int d = 0; d < 3; ++d) {
        const double e = g->origin[d] + h[d] * (double)g->res[d];
        lo[d] = std::min(g->origin[d], e);
        hi[d] = std::max(g->origin[d], e);
    }
    const unsigned nsub = (unsigned)std::max(max_cfl, 1.0);
    const double sdt = dt / nsub;
    auto mat = [](const double* m, const double v[3], double o[3]) {
        o[0] = m[0] * v[0] + m[1] * v[1] + m[2] * v[2];
        o[1] = m[3] * v[0] + m[4] * v[1] + m[5] * v[2];
        o[2] = m[6] * v[0] + m[7] * v[1] + m[8] * v[2];
    };
#pragma omp parallel for schedule(static)
    for (long q = 0; q < np; ++q) {
        double p0[3] = {pos[3 * q], pos[3 * q + 1], pos[3 * q + 2]};
        double p1[3] = {p0[0], p0[1], p0[2]};
        double vv[3] = {vel[3 * q], vel[3 * q + 1], vel[3 * q + 2]};
        for (unsigned t = 0; t < nsub; ++t) {
            double v0[3], mid[3], vm[3];
            sample(p0, v0);
            const double hs = 0.5 * sdt;
            for (int d = 0; d < 3; ++d) mid[d] = p0[d] + hs * v0[d];
            sample(mid, vm);
            for (int d = 0; d < 3; ++d) p1[d] = p0[d] + sdt * vm[d];
            for (int d = 0; d < 3; ++d) p0[d] = p1[d];
        }
        for (int d = 0; d < 3; ++d) {
            if ((closed & (1 << (2 * d))) && p1[d] <= lo[d]) {
                p1[d] = lo[d];
                vv[d] = 0.0;
            }
            if ((closed & (1 << (2 * d + 1))) && p1[d] >= hi[d]) {
                p1[d] = hi[d];
                vv[d] = 0.0;
            }
        }
        if (col && sph) {
            // World -> local: inverse orientation of (p - translation).
            const double* t = col->centre;
            const double dp[3] = {p1[0] - t[0], p1[1] - t[1], p1[2] - t[2]};
            double pl[3];
            mat(sph->inv_orient, dp, pl);
            const double* c = sph->center;
            // closestNormalLocal (sphere3.cpp:33-39).
            double nl[3];
            if (std::fabs(c[0] - pl[0]) < kEpsD &&
                std::fabs(c[1] - pl[1]) < kEpsD &&
                std::fabs(c[2] - pl[2]) < kEpsD) {
                nl[0] = 1;
                nl[1] = 0;
                nl[2] = 0;
            } else {
                const double dd[3] = {pl[0] - c[0], pl[1] - c[1], pl[2] - c[2]};
                const double l = std::sqrt(dd[0] * dd[0] + dd[1] * dd[1] +
                                           dd[2] * dd[2]);
                nl[0] = dd[0] / l;
                nl[1] = dd[1] / l;
                nl[2] = dd[2] / l;
            }
            const double r = sph->radius;
            const double cpl[3] = {r * nl[0] + c[0], r * nl[1] + c[1],
                                   r * nl[2] + c[2]};
            // closestDistanceLocal (sphere3.cpp:29-31).
            const double e3[3] = {c[0] - pl[0], c[1] - pl[1], c[2] - pl[2]};
            const double dist = std::fabs(
                std::sqrt(e3[0] * e3[0] + e3[1] * e3[1] + e3[2] * e3[2]) - r);
            // isInsideLocal (surface3.cpp:75-79) and isInside (:67-69).
            const double off[3] = {pl[0] - cpl[0], pl[1] - cpl[1],
                                   pl[2] - cpl[2]};
            const bool inLocal =
                off[0] * nl[0] + off[1] * nl[1] + off[2] * nl[2] < 0.0;
            const bool isIn = (sph->normal_flipped != 0) == !inLocal;
            if (isIn || dist < 0.0) {
                // closestPoint / closestNormal in world space.
                double cpw[3], nw[3];
                mat(sph->orient, cpl, cpw);
                for (int d = 0; d < 3; ++d) cpw[d] = cpw[d] + t[d];
                mat(sph->orient, nl, nw);
                const double fl = sph->normal_flipped ? -1.0 : 1.0;
                for (int d = 0; d < 3; ++d) nw[d] *= fl;
                // velocityAt(query point) (rigid_body_collider3.cpp:25-28).
                const double* a = col->ang;
                const double rr[3] = {p1[0] - t[0], p1[1] - t[1], p1[2] - t[2]};
                const double cv[3] = {
                    col->lin[0] + (a[1] * rr[2] - rr[1] * a[2]),
                    col->lin[1] + (a[2] * rr[0] - rr[2] * a[0]),
                    col->lin[2] + (a[0] * rr[1] - rr[0] * a[1])};
                double tp[3];
                for (int d = 0; d < 3; ++d) tp[d] = cpw[d] + 0.0 * nw[d];
                const double rv[3] = {vv[0] - cv[0], vv[1] - cv[1],
                                      vv[2] - cv[2]};
                const double ndv = nw[0] * rv[0] + nw[1] * rv[1] + nw[2] * rv[2];
                double rn[3] = {ndv * nw[0], ndv * nw[1], ndv * nw[2]};
                double rt[3] = {rv[0] - rn[0], rv[1] - rn[1], rv[2] - rn[2]};
                if (ndv < 0.0) {
                    const double rest = 0.0;
                    const double dn[3] = {(-rest - 1.0) * rn[0],
                                          (-rest - 1.0) * rn[1],
                                          (-rest - 1.0) * rn[2]};
                    for (int d = 0; d < 3; ++d) rn[d] *= -rest;
                    const double lt2 = rt[0] * rt[0] + rt[1] * rt[1] + rt[2] * rt[2];
                    if (lt2 > 0.0) {
                        const double ldn = std::sqrt(dn[0] * dn[0] + dn[1] * dn[1] +
                                                     dn[2] * dn[2]);
                        const double fs = std::max(
                            1.0 - col->friction * ldn / std::sqrt(lt2), 0.0);
                        for (int d = 0; d < 3; ++d) rt[d] *= fs;
                    }
                    for (int d = 0; d < 3; ++d) vv[d] = rn[d] + rt[d] + cv[d];
                }
                for (int d = 0; d < 3; ++d) p1[d] = tp[d];
            }
        }
        for (int d = 0; d < 3; ++d) {
            pos[3 * q + d] = p1[d];
            vel[3 * q + d] = vv[d];
        }
    }
}

// PicSolver3::buildSignedDistanceField (src/jet/pic_solver3.cpp:296-317) and
// GridFluidSolver3::extrapolateIntoCollider (grid_fluid_solver3.cpp:423-438).
// The reference's hash-grid search visits exactly the particles whose
// squared distance (x - p).(x - p) is <= band^2, and takes the minimum of
// their distances, so any search that finds that set gives the same value;
// this one bins particles into cells of the band size.
void orc_build_particle_sdf(const orc_grid* g, long np, const double* pos,
                            const orc_field* collider_sdf, double max_cfl,
                            double* out) {
    const Size3 s{g->res[0], g->res[1], g->res[2]};
    const double* h = g->spacing;
    const double maxH = std::max(std::max(h[0], h[1]), h[2]);
    const double radius = 1.2 * maxH / std::sqrt(2.0);
    const double band = 2.0 * radius;
    const double band2 = band * band;
    const double o[3] = {g->origin[0] + 0.5 * h[0], g->origin[1] + 0.5 * h[1],
                         g->origin[2] + 0.5 * h[2]};
    // Bins of edge `band` over the particles' bounding box.
    double lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
    long nb[3] = {1, 1, 1};
    std::vector<long> start, order;
    auto binOf = [&](const double* p, long* b) {
        for (int d = 0; d < 3; ++d) {
            double f = std::floor((p[d] - lo[d]) / band);
            if (!(f >= 0)) f = 0;
            if (f > nb[d] - 1) f = (double)(nb[d] - 1);
            b[d] = (long)f;
        }
    };
    if (np > 0) {
        for (int d = 0; d < 3; ++d) {
            lo[d] = hi[d] = pos[d];
            for (long q = 1; q < np; ++q) {
                lo[d] = std::min(lo[d], pos[3 * q + d]);
                hi[d] = std::max(hi[d], pos[3 * q + d]);
            }
            nb[d] = std::max(1L, std::min(1L << 20, (long)((hi[d] - lo[d]) / band) + 1));
        }
        const long nbin = nb[0] * nb[1] * nb[2];
        std::vector<long> cnt(nbin + 1, 0), key(np);
        for (long q = 0; q < np; ++q) {
            long b[3];
            binOf(pos + 3 * q, b);
            key[q] = b[0] + nb[0] * (b[1] + nb[1] * b[2]);
            ++cnt[key[q] + 1];
        }
        for (long b = 0; b < nbin; ++b) cnt[b + 1] += cnt[b];
        start = cnt;
        order.resize(np);
        for (long q = 0; q < np; ++q) order[cnt[key[q]]++] = q;
    }
#pragma omp parallel for schedule(static)
    for (long k = 0; k < s.z; ++k)
        for (long j = 0; j < s.y; ++j)
            for (long i = 0; i < s.x; ++i) {
                const double pt[3] = {o[0] + h[0] * (double)i,
                                      o[1] + h[1] * (double)j,
                                      o[2] + h[2] * (double)k};
                double minDist = band;
                if (np > 0) {
                    long b0[3], b1[3];
                    const double plo[3] = {pt[0] - band, pt[1] - band, pt[2] - band};
                    const double phi[3] = {pt[0] + band, pt[1] + band, pt[2] + band};
                    binOf(plo, b0);
                    binOf(phi, b1);
                    for (long bz = b0[2]; bz <= b1[2]; ++bz)
                        for (long by = b0[1]; by <= b1[1]; ++by)
                            for (long bx = b0[0]; bx <= b1[0]; ++bx) {
                                const long b = bx + nb[0] * (by + nb[1] * bz);
                                for (long e = start[b]; e < start[b + 1]; ++e) {
                                    const double* x = pos + 3 * order[e];
                                    const double d0 = x[0] - pt[0], d1 = x[1] - pt[1],
                                                 d2 = x[2] - pt[2];
                                    if (d0 * d0 + d1 * d1 + d2 * d2 <= band2) {
                                        const double e0 = pt[0] - x[0], e1 = pt[1] - x[1],
                                                     e2 = pt[2] - x[2];
                                        const double dist =
                                            std::sqrt(e0 * e0 + e1 * e1 + e2 * e2);
                                        minDist = std::min(minDist, dist);
                                    }
                                }
                            }
                }
                out[lin(s, i, j, k)] = minDist - radius;
            }
    // extrapolateIntoCollider: valid where the collider SDF is not negative.
    Field C{collider_sdf};
    std::vector<char> valid(s.count());
#pragma omp parallel for schedule(static)
    for (long k = 0; k < s.z; ++k)
        for (long j = 0; j < s.y; ++j)
            for (long i = 0; i < s.x; ++i)
                valid[lin(s, i, j, k)] =
                    inside(C.sample(o[0] + h[0] * (double)i, o[1] + h[1] * (double)j,
                                    o[2] + h[2] * (double)k)) ? 0 : 1;
    const int res[3] = {(int)s.x, (int)s.y, (int)s.z};
    orc_extrapolate(res, out, valid.data(), (unsigned)std::ceil(max_cfl));
}

// The bounding box and half spacing ApicSolver3 clamps positions with
// (apic_solver3.cpp:33-34), and jet::clamp (math_utils-inl.h:126-134).
struct ApicFrame {
    double lo[3], hi[3], hh[3];
};
ApicFrame apicFrame(const orc_grid* g) {
    ApicFrame f;
    for (int d = 0; d < 3; ++d) {
        const double e = g->origin[d] + g->spacing[d] * (double)g->res[d];
        f.lo[d] = std::min(g->origin[d], e);
        f.hi[d] = std::max(g->origin[d], e);
        f.hh[d] = g->spacing[d] / 2.0;
    }
    return f;
}
inline double clampd(double v, double lo, double hi) {
    return v < lo ? lo : (v > hi ? hi : v);
}
// The position clamped for face grid a: the two other coordinates kept half
// a cell inside the box.
inline void apicClamp(const ApicFrame& f, int a, const double* p, double q[3]) {
    for (int d = 0; d < 3; ++d)
        q[d] = d == a ? p[d] : clampd(p[d], f.lo[d] + f.hh[d], f.hi[d] - f.hh[d]);
}

void orc_apic_p2g(const orc_grid* g, long np, const double* pos,
                  const double* vel, const double* affine, double* u,
                  double* v, double* w, char* mu, char* mv, char* mw) {
    FaceGeom fg[3];
    faceGeoms(g, fg);
    const ApicFrame F = apicFrame(g);
    const double* h = g->spacing;
    double* grids[3] = {u, v, w};
    char* marks[3] = {mu, mv, mw};
    std::vector<double> wsum[3];
    for (int a = 0; a < 3; ++a) {
        const long n = fg[a].s.count();
        std::fill(grids[a], grids[a] + n, 0.0);
        wsum[a].assign(n, 0.0);
        if (marks[a]) std::fill(marks[a], marks[a] + n, 0);
    }
    for (long p = 0; p < np; ++p) {  // serial, in index order
        for (int a = 0; a < 3; ++a) {
            double q[3];
            apicClamp(F, a, pos + 3 * p, q);
            Stencil st;
            coordsAndWeights(fg[a].s, fg[a].o[0], fg[a].o[1], fg[a].o[2],
                             1.0 / h[0], 1.0 / h[1], 1.0 / h[2], q[0], q[1],
                             q[2], &st);
            const double* C = affine + 9 * p + 3 * a;
            const Size3 s = fg[a].s;
            for (int n = 0; n < 8; ++n) {
                const long c = st.idx[n];
                const long i = c % s.x, j = (c / s.x) % s.y, k = c / (s.x * s.y);
                const double gp[3] = {fg[a].o[0] + h[0] * (double)i,
                                      fg[a].o[1] + h[1] * (double)j,
                                      fg[a].o[2] + h[2] * (double)k};
                const double term = C[0] * (gp[0] - q[0]) +
                                    C[1] * (gp[1] - q[1]) +
                                    C[2] * (gp[2] - q[2]);
                grids[a][c] += st.w[n] * (vel[3 * p + a] + term);
                wsum[a][c] += st.w[n];
                if (marks[a]) marks[a][c] = 1;
            }
        }
    }
    for (int a = 0; a < 3; ++a)
        for (long c = 0; c < fg[a].s.count(); ++c)
            if (wsum[a][c] > 0.0) grids[a][c] /= wsum[a][c];
}

void orc_apic_g2p(const orc_grid* g, long np, const double* pos, double* vel,
                  double* affine, const double* u, const double* v,
                  const double* w) {
    FaceGeom fg[3];
    faceGeoms(g, fg);
    const ApicFrame F = apicFrame(g);
    const double* h = g->spacing;
    const double* grids[3] = {u, v, w};
    const double ih[3] = {1.0 / h[0], 1.0 / h[1], 1.0 / h[2]};
#pragma omp parallel for schedule(static)
    for (long p = 0; p < np; ++p) {
        for (int a = 0; a < 3; ++a) {  // velocities[i] = flow->sample(x)
            const double nx = (pos[3 * p] - fg[a].o[0]) / h[0];
            const double ny = (pos[3 * p + 1] - fg[a].o[1]) / h[1];
            const double nz = (pos[3 * p + 2] - fg[a].o[2]) / h[2];
            vel[3 * p + a] = trilinear<double, double>(grids[a], fg[a].s, nx, ny, nz);
        }
        for (int a = 0; a < 3; ++a) {
            double q[3];
            apicClamp(F, a, pos + 3 * p, q);
            // getCoordinatesAndGradientWeights (array_samplers3-inl.h:196-261).
            const Size3 s = fg[a].s;
            long i, j, k;
            double fx, fy, fz;
            barycentric<double>((q[0] - fg[a].o[0]) / h[0], s.x - 1, &i, &fx);
            barycentric<double>((q[1] - fg[a].o[1]) / h[1], s.y - 1, &j, &fy);
            barycentric<double>((q[2] - fg[a].o[2]) / h[2], s.z - 1, &k, &fz);
            const long ip1 = std::min(i + 1, s.x - 1), jp1 = std::min(j + 1, s.y - 1),
                       kp1 = std::min(k + 1, s.z - 1);
            const long idx[8] = {lin(s, i, j, k),     lin(s, ip1, j, k),
                                 lin(s, i, jp1, k),   lin(s, ip1, jp1, k),
                                 lin(s, i, j, kp1),   lin(s, ip1, j, kp1),
                                 lin(s, i, jp1, kp1), lin(s, ip1, jp1, kp1)};
            const double ix = ih[0], iy = ih[1], iz = ih[2];
            const double gw[8][3] = {
                {-ix * (1 - fy) * (1 - fz), -iy * (1 - fx) * (1 - fz), -iz * (1 - fx) * (1 - fy)},
                {ix * (1 - fy) * (1 - fz), fx * (-iy) * (1 - fz), fx * (1 - fy) * (-iz)},
                {(-ix) * fy * (1 - fz), (1 - fx) * iy * (1 - fz), (1 - fx) * fy * (-iz)},
                {ix * fy * (1 - fz), fx * iy * (1 - fz), fx * fy * (-iz)},
                {(-ix) * (1 - fy) * fz, (1 - fx) * (-iy) * fz, (1 - fx) * (1 - fy) * iz},
                {ix * (1 - fy) * fz, fx * (-iy) * fz, fx * (1 - fy) * iz},
                {(-ix) * fy * fz, (1 - fx) * iy * fz, (1 - fx) * fy * iz},
                {ix * fy * fz, fx * iy * fz, fx * fy * iz}};
            double C[3] = {0.0, 0.0, 0.0};
            for (int n = 0; n < 8; ++n) {
                const double val = grids[a][idx[n]];
                for (int d = 0; d < 3; ++d) C[d] = C[d] + gw[n][d] * val;
            }
            for (int d = 0; d < 3; ++d) affine[9 * p + 3 * a + d] = C[d];
        }
    }
}

// extrapolateToRegion (include/jet/detail/array_utils-inl.h:172-244). An
// iteration writes only cells invalid at its start and reads only cells
// valid at its start, so it is order-independent.
void orc_extrapolate(const int res[3], double* data, const char* valid,
                     unsigned int iterations) {
    const Size3 s{res[0], res[1], res[2]};
    std::vector<char> v0(valid, valid + s.count()), v1(s.count(), 0);
    for (unsigned it = 0; it < iterations; ++it) {
#pragma omp parallel for schedule(static)
        for (long k = 0; k < s.z; ++k)
            for (long j = 0; j < s.y; ++j)
                for (long i = 0; i < s.x; ++i) {
                    const long c = lin(s, i, j, k);
                    if (v0[c]) {
                        v1[c] = 1;
                        continue;
                    }
                    double sum = 0.0;
                    unsigned count = 0;
                    auto take = [&](bool ok, long n) {
                        if (ok && v0[n]) {
                            sum += data[n];
                            ++count;
                        }
                    };
                    take(i + 1 < s.x, c + 1);
                    take(i > 0, c - 1);
                    take(j + 1 < s.y, c + s.x);
                    take(j > 0, c - s.x);
                    take(k + 1 < s.z, c + s.x * s.y);
                    take(k > 0, c - s.x * s.y);
                    if (count > 0) {
                        data[c] = sum / (double)count;
                        v1[c] = 1;
                    } else {
                        v1[c] = 0;
                    }
                }
        v0.swap(v1);
    }
}

void orc_g2p_pic(const orc_grid* g, long np, const double* pos, double* vel,
                 const double* u, const double* v, const double* w) {
    FaceGeom fg[3];
    faceGeoms(g, fg);
    const double* grids[3] = {u, v, w};
#pragma omp parallel for schedule(static)
    for (long p = 0; p < np; ++p) {
        for (int a = 0; a < 3; ++a) {
            double nx = (pos[3 * p] - fg[a].o[0]) / g->spacing[0];
            double ny = (pos[3 * p + 1] - fg[a].o[1]) / g->spacing[1];
            double nz = (pos[3 * p + 2] - fg[a].o[2]) / g->spacing[2];
            vel[3 * p + a] =
                trilinear<double, double>(grids[a], fg[a].s, nx, ny, nz);
        }
    }
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Blocked pressure solver (src/jet/grid_single_phase_pressure_solver3.cpp)
// with an FdmMgpcgSolver3 installed: cells are marked fluid, air or boundary
// at their centres, coarse levels take the majority marker of a 4x4x4 block,
// and every level's matrix is the 7-point Laplacian on those markers.

namespace {

constexpr char kMFluid = 0, kMAir = 1, kMBoundary = 2;

struct BlockedState {
    std::vector<Size3> sizes;
    std::vector<std::vector<char>> markers;
    std::vector<Level> levels;
};

BlockedState g_blocked;

// argmax3 (include/jet/detail/math_utils-inl.h:106-113).
inline int argmax3i(int x, int y, int z) {
    if (x > y) return (x > z) ? 0 : 2;
    return (y > z) ? 1 : 2;
}

// buildMarkers (:245-322).
void blockedMarkers(const orc_grid* g, const orc_field* bsdf,
                    const orc_field* fsdf, unsigned maxLevels) {
    BlockedState& S = g_blocked;
    Size3 n{g->res[0], g->res[1], g->res[2]};
    S.sizes = levelSizes(n, maxLevels);
    S.markers.assign(S.sizes.size(), {});
    for (size_t l = 0; l < S.sizes.size(); ++l)
        S.markers[l].assign(S.sizes[l].count(), kMFluid);
    Field B{bsdf}, F{fsdf};
    std::vector<char>& m0 = S.markers[0];
    const double hx = g->spacing[0], hy = g->spacing[1], hz = g->spacing[2];
    const double ox = g->origin[0], oy = g->origin[1], oz = g->origin[2];
#pragma omp parallel for schedule(static)
    for (long k = 0; k < n.z; ++k)
        for (long j = 0; j < n.y; ++j)
            for (long i = 0; i < n.x; ++i) {
                // Grid3::cellCenterPosition (src/jet/grid3.cpp:32-38).
                const double x = ox + hx * ((double)i + 0.5);
                const double y = oy + hy * ((double)j + 0.5);
                const double z = oz + hz * ((double)k + 0.5);
                char m;
                if (inside(B.sample(x, y, z)))
                    m = kMBoundary;
                else if (inside(F.sample(x, y, z)))
                    m = kMFluid;
                else
                    m = kMAir;
                m0[lin(n, i, j, k)] = m;
            }
    for (size_t l = 1; l < S.sizes.size(); ++l) {
        const Size3 f = S.sizes[l - 1], c = S.sizes[l];
        const std::vector<char>& fine = S.markers[l - 1];
        std::vector<char>& coarse = S.markers[l];
#pragma omp parallel for schedule(static)
        for (long k = 0; k < c.z; ++k)
            for (long j = 0; j < c.y; ++j)
                for (long i = 0; i < c.x; ++i) {
                    const long kI[4] = {k > 0 ? 2 * k - 1 : 2 * k, 2 * k,
                                        2 * k + 1,
                                        k + 1 < c.z ? 2 * k + 2 : 2 * k + 1};
                    const long jI[4] = {j > 0 ? 2 * j - 1 : 2 * j, 2 * j,
                                        2 * j + 1,
                                        j + 1 < c.y ? 2 * j + 2 : 2 * j + 1};
                    const long iI[4] = {i > 0 ? 2 * i - 1 : 2 * i, 2 * i,
                                        2 * i + 1,
                                        i + 1 < c.x ? 2 * i + 2 : 2 * i + 1};
                    int cnt[3] = {0, 0, 0};
                    for (int z = 0; z < 4; ++z)
                        for (int y = 0; y < 4; ++y)
                            for (int x = 0; x < 4; ++x) {
                                const char v = fine[lin(f, iI[x], jI[y], kI[z])];
                                if (v == kMBoundary)
                                    ++cnt[2];
                                else if (v == kMFluid)
                                    ++cnt[0];
                                else
                                    ++cnt[1];
                            }
                    coarse[lin(c, i, j, k)] =
                        (char)argmax3i(cnt[0], cnt[1], cnt[2]);
                }
    }
}

// buildSingleSystem, FdmMatrix3 form (:26-76). `u` is NULL on coarse levels,
// whose right-hand sides the multigrid overwrites by restriction
// (include/jet/detail/mg-inl.h:28-30); b stays zero there.
void blockedSystem(Level& L, const std::vector<char>& m, double hx, double hy,
                   double hz, const double* u, const double* v,
                   const double* w) {
    const Size3 n = L.size;
    L.A.assign(n.count(), Row{0, 0, 0, 0});
    L.b.assign(n.count(), 0.0);
    L.x.assign(n.count(), 0.0);
    const double ihx = 1.0 / hx, ihy = 1.0 / hy, ihz = 1.0 / hz;
    const double isx = ihx * ihx, isy = ihy * ihy, isz = ihz * ihz;
    const Size3 us{n.x + 1, n.y, n.z}, vs{n.x, n.y + 1, n.z},
        ws{n.x, n.y, n.z + 1};
    const long sy = n.x, sz = n.x * n.y;
#pragma omp parallel for schedule(static)
    for (long k = 0; k < n.z; ++k)
        for (long j = 0; j < n.y; ++j)
            for (long i = 0; i < n.x; ++i) {
                const long c = lin(n, i, j, k);
                Row& r = L.A[c];
                if (m[c] != kMFluid) {
                    r.center = 1.0;
                    continue;
                }
                if (u) {
                    // FaceCenteredGrid3::divergenceAtCellCenter
                    // (src/jet/face_centered_grid3.cpp:137-152).
                    const double du = u[lin(us, i + 1, j, k)] - u[lin(us, i, j, k)];
                    const double dv = v[lin(vs, i, j + 1, k)] - v[lin(vs, i, j, k)];
                    const double dw = w[lin(ws, i, j, k + 1)] - w[lin(ws, i, j, k)];
                    L.b[c] = du / hx + dv / hy + dw / hz;
                }
                if (i + 1 < n.x && m[c + 1] != kMBoundary) {
                    r.center += isx;
                    if (m[c + 1] == kMFluid) r.right -= isx;
                }
                if (i > 0 && m[c - 1] != kMBoundary) r.center += isx;
                if (j + 1 < n.y && m[c + sy] != kMBoundary) {
                    r.center += isy;
                    if (m[c + sy] == kMFluid) r.up -= isy;
                }
                if (j > 0 && m[c - sy] != kMBoundary) r.center += isy;
                if (k + 1 < n.z && m[c + sz] != kMBoundary) {
                    r.center += isz;
                    if (m[c + sz] == kMFluid) r.front -= isz;
                }
                if (k > 0 && m[c - sz] != kMBoundary) r.center += isz;
            }
}

// applyPressureGradient (:378-405): only the +x/+y/+z faces of fluid cells
// whose neighbour is not a boundary cell change; out_* start as copies of
// the input.
void blockedGradient(const orc_grid* g, const double* x, const double* u,
                     const double* v, const double* w, double* ou,
                     double* ov, double* ow) {
    const std::vector<char>& m = g_blocked.markers[0];
    const Size3 n{g->res[0], g->res[1], g->res[2]};
    const Size3 us{n.x + 1, n.y, n.z}, vs{n.x, n.y + 1, n.z},
        ws{n.x, n.y, n.z + 1};
    const double ihx = 1.0 / g->spacing[0], ihy = 1.0 / g->spacing[1],
                 ihz = 1.0 / g->spacing[2];
    const long sy = n.x, sz = n.x * n.y;
#pragma omp parallel for schedule(static)
    for (long k = 0; k < n.z; ++k)
        for (long j = 0; j < n.y; ++j)
            for (long i = 0; i < n.x; ++i) {
                const long c = lin(n, i, j, k);
                if (m[c] != kMFluid) continue;
                if (i + 1 < n.x && m[c + 1] != kMBoundary) {
                    const long f = lin(us, i + 1, j, k);
                    ou[f] = u[f] + ihx * (x[c + 1] - x[c]);
                }
                if (j + 1 < n.y && m[c + sy] != kMBoundary) {
                    const long f = lin(vs, i, j + 1, k);
                    ov[f] = v[f] + ihy * (x[c + sy] - x[c]);
                }
                if (k + 1 < n.z && m[c + sz] != kMBoundary) {
                    const long f = lin(ws, i, j, k + 1);
                    ow[f] = w[f] + ihz * (x[c + sz] - x[c]);
                }
            }
}

}  // namespace

extern "C" {

int orc_blocked_pressure_solve(const orc_grid* g, const double* u,
                               const double* v, const double* w,
                               const orc_field* boundary_sdf,
                               const orc_field* fluid_sdf,
                               const orc_mg_params* p, double* out_u,
                               double* out_v, double* out_w, double* out_p,
                               unsigned int* iters, double* resid) {
    BlockedState& S = g_blocked;
    blockedMarkers(g, boundary_sdf, fluid_sdf, p->max_levels);
    const size_t nl = S.sizes.size();
    S.levels.assign(nl, {});
    // buildSystem (:341-376): coarse levels use the doubled spacing.
    double hx = g->spacing[0], hy = g->spacing[1], hz = g->spacing[2];
    for (size_t l = 0; l < nl; ++l) {
        if (l > 0) {
            hx *= 2.0;
            hy *= 2.0;
            hz *= 2.0;
        }
        S.levels[l].size = S.sizes[l];
        blockedSystem(S.levels[l], S.markers[l], hx, hy, hz,
                      l == 0 ? u : nullptr, l == 0 ? v : nullptr,
                      l == 0 ? w : nullptr);
    }
    MgSolver solver{*p, &S.levels, {}, {}, {}};
    unsigned it = 0;
    double rs = 0;
    const bool ok = solver.solve(&it, &rs);
    if (iters) *iters = it;
    if (resid) *resid = rs;
    const Size3 n{g->res[0], g->res[1], g->res[2]};
    const long nu = (n.x + 1) * n.y * n.z, nv = n.x * (n.y + 1) * n.z,
               nw = n.x * n.y * (n.z + 1);
    std::vector<double> cu(u, u + nu), cv(v, v + nv), cw(w, w + nw);
    if (out_u != u) std::memcpy(out_u, u, nu * sizeof(double));
    if (out_v != v) std::memcpy(out_v, v, nv * sizeof(double));
    if (out_w != w) std::memcpy(out_w, w, nw * sizeof(double));
    blockedGradient(g, S.levels[0].x.data(), cu.data(), cv.data(), cw.data(),
                    out_u, out_v, out_w);
    if (out_p)
        std::memcpy(out_p, S.levels[0].x.data(), n.count() * sizeof(double));
    return ok ? 1 : 0;
}

long orc_blocked_get_level(int level, int what, void* dst) {
    BlockedState& S = g_blocked;
    if (level < 0 || level >= (int)S.levels.size()) return -1;
    const Level& L = S.levels[level];
    switch (what) {
        case 0:
            std::memcpy(dst, S.markers[level].data(), S.markers[level].size());
            return (long)S.markers[level].size();
        case 4:
            std::memcpy(dst, L.A.data(), L.A.size() * sizeof(Row));
            return (long)L.A.size();
        case 5:
            std::memcpy(dst, L.b.data(), L.b.size() * sizeof(double));
            return (long)L.b.size();
        default:
            return -1;
    }
}

}  // extern "C"

extern "C" {

// GridBlockedBoundaryConditionSolver3::constrainVelocity
// (src/jet/grid_blocked_boundary_condition_solver3.cpp:23-67): the
// fractional constraint, then every face between a collider cell (collider
// SDF sample < 0 at the cell, :79-90) and a non-collider neighbour takes the
// collider velocity's normal component at the face position. Each such face
// has one collider side, so the pass is order-independent.
void orc_constrain_velocity_blocked(const orc_grid* g, double* u, double* v,
                                    double* w, const orc_field* sdf,
                                    const orc_collider* col, int closed,
                                    unsigned int depth) {
    orc_constrain_velocity(g, u, v, w, sdf, col, closed, depth);
    const Size3 n{g->res[0], g->res[1], g->res[2]};
    const Size3 us{n.x + 1, n.y, n.z}, vs{n.x, n.y + 1, n.z},
        ws{n.x, n.y, n.z + 1};
    const double* h = g->spacing;
    FaceGeom fg[3];
    faceGeoms(g, fg);
    auto solid = [&](long i, long j, long k) {
        const double phi = sdf->kind == 1 ? sdf->data[lin(n, i, j, k)]
                                          : sdf->value;
        return inside(phi);
    };
    // RigidBodyCollider3::velocityAt (rigid_body_collider3.cpp:25-28).
    auto colVel = [&](const double p[3], int a) {
        if (col == nullptr) return 0.0;
        const double* an = col->ang;
        const double r[3] = {p[0] - col->centre[0], p[1] - col->centre[1],
                             p[2] - col->centre[2]};
        const double cr[3] = {an[1] * r[2] - r[1] * an[2],
                              an[2] * r[0] - r[2] * an[0],
                              an[0] * r[1] - r[0] * an[1]};
        return col->lin[a] + cr[a];
    };
    // uPosition/vPosition/wPosition (src/jet/face_centered_grid3.cpp:
    // 216-238): the face array's data origin + spacing * (i, j, k).
    auto pos = [&](int a, long i, long j, long k, double p[3]) {
        p[0] = fg[a].o[0] + h[0] * (double)i;
        p[1] = fg[a].o[1] + h[1] * (double)j;
        p[2] = fg[a].o[2] + h[2] * (double)k;
    };
#pragma omp parallel for schedule(static)
    for (long k = 0; k < n.z; ++k)
        for (long j = 0; j < n.y; ++j)
            for (long i = 0; i < n.x; ++i) {
                if (!solid(i, j, k)) continue;
                double p[3];
                if (i > 0 && !solid(i - 1, j, k)) {
                    pos(0, i, j, k, p);
                    u[lin(us, i, j, k)] = colVel(p, 0);
                }
                if (i < n.x - 1 && !solid(i + 1, j, k)) {
                    pos(0, i + 1, j, k, p);
                    u[lin(us, i + 1, j, k)] = colVel(p, 0);
                }
                if (j > 0 && !solid(i, j - 1, k)) {
                    pos(1, i, j, k, p);
                    v[lin(vs, i, j, k)] = colVel(p, 1);
                }
                if (j < n.y - 1 && !solid(i, j + 1, k)) {
                    pos(1, i, j + 1, k, p);
                    v[lin(vs, i, j + 1, k)] = colVel(p, 1);
                }
                if (k > 0 && !solid(i, j, k - 1)) {
                    pos(2, i, j, k, p);
                    w[lin(ws, i, j, k)] = colVel(p, 2);
                }
                if (k < n.z - 1 && !solid(i, j, k + 1)) {
                    pos(2, i, j, k + 1, p);
                    w[lin(ws, i, j, k + 1)] = colVel(p, 2);
                }
            }
}

}  // extern "C"
