// Seeded synthetic bundle-adjustment problems (see include/nav_ba_synth.h).
//
// Camera convention (OpenCV / nav24): x right, y down, z forward; a pose is T_cw with
// X_c = R_cw X_w + t_cw.  Observations are generated from the true geometry plus pixel noise;
// initial estimates are the true ones perturbed (fixed cameras are left at the truth, they
// carry the gauge).  Observations come out point-major, cameras ascending within a point,
// which is the edge order nav24's graph build produces for one point (BE_GraphOptim.cpp:156-199).
#include "../../include/nav_ba_synth.h"

#include <algorithm>
#include <array>
#include <cmath>
#include <cstring>
#include <random>
#include <unordered_map>
#include <vector>

namespace {

constexpr double kPi = 3.14159265358979323846;
constexpr double kFx = 500.0, kFy = 500.0, kCx = 320.0, kCy = 240.0;
constexpr double kWidth = 640.0, kHeight = 480.0;

using Vec3 = std::array<double, 3>;
using Mat3 = std::array<double, 9>;  // row-major

// Host-independent elementary functions.  The platform libm may pick a different sin/cos/log per
// CPU (glibc on x86-64 selects an FMA variant at run time), which changes last bits and, through
// the visibility tests, the whole random stream.  These use only +, -, *, / and sqrt, all
// correctly rounded in IEEE double, and the file is compiled without contraction, so every host
// produces the same bits.  Accuracy is a few ulp, which is all the generator needs.
//
// sin/cos: Cody-Waite reduction x = k*pi/2 + r with pi/2 split into a 32-bit head (k*head exact for
// |k| < 2^21) and a tail, then the Taylor series of sin and cos on |r| <= pi/4 to order 17/18
// (remainder below 1e-19), nested so each step divides by the next factorial ratio.
struct PiHalf {
    double head, tail;
    PiHalf() {
        const double ph = 1.5707963267948966;  // pi/2 rounded to double
        uint64_t b;
        std::memcpy(&b, &ph, 8);
        b &= ~((uint64_t(1) << 21) - 1);       // keep 32 significant bits
        std::memcpy(&head, &b, 8);
        tail = (ph - head) + 6.123233995736766e-17;  // pi/2 - double(pi/2) = 6.1232339957367658e-17
    }
};
const PiHalf kPiHalf;

void dsincos(double x, double* s, double* c) {
    const double kd = std::nearbyint(x * (2.0 / kPi));
    const double r = (x - kd * kPiHalf.head) - kd * kPiHalf.tail;
    const double r2 = r * r;
    double ps = 1.0, pc = 1.0;
    for (int n = 9; n >= 1; --n) {  // sin: 1 - r2/(2n(2n+1)) (...);  cos: 1 - r2/((2n-1)2n) (...)
        ps = 1.0 - r2 / (double)((2 * n) * (2 * n + 1)) * ps;
        pc = 1.0 - r2 / (double)((2 * n - 1) * (2 * n)) * pc;
    }
    const double sr = r * ps, cr = pc;
    switch (((long long)kd % 4 + 4) % 4) {
        case 0: *s = sr; *c = cr; break;
        case 1: *s = cr; *c = -sr; break;
        case 2: *s = -sr; *c = -cr; break;
        default: *s = -cr; *c = sr; break;
    }
}
double dsin(double x) { double s, c; dsincos(x, &s, &c); return s; }
double dcos(double x) { double s, c; dsincos(x, &s, &c); return c; }

// log for x > 0: x = m 2^e with m in [sqrt(1/2), sqrt(2)) (frexp is exact), log m = 2 atanh(t) with
// t = (m-1)/(m+1), |t| <= 0.1716, by its series t + t^3/3 + ... to t^25 (remainder below 1e-20);
// ln 2 as a double plus its rounding error.
double dlog(double x) {
    int e;
    double m = std::frexp(x, &e);
    if (m < 0.70710678118654752) { m *= 2.0; e -= 1; }
    const double t = (m - 1.0) / (m + 1.0), t2 = t * t;
    double p = 1.0 / 25.0;
    for (int k = 11; k >= 0; --k) p = 1.0 / (double)(2 * k + 1) + t2 * p;
    return (double)e * 0.6931471805599453 + ((double)e * 2.3190468138462996e-17 + 2.0 * t * p);
}

// Deterministic random source: mt19937_64 bits, uniform from the top 53 bits, normal by the
// Box-Muller transform (Box & Muller 1958).
struct Rng {
    std::mt19937_64 g;
    bool has_spare = false;
    double spare = 0.0;
    explicit Rng(uint64_t seed) : g(seed) {}
    double uniform() { return (double)(g() >> 11) * (1.0 / 9007199254740992.0); }
    double uniform(double lo, double hi) { return lo + (hi - lo) * uniform(); }
    int uniform_int(int lo, int hi) {  // inclusive
        return lo + (int)(uniform() * (double)(hi - lo + 1)) % (hi - lo + 1);
    }
    double normal() {
        if (has_spare) { has_spare = false; return spare; }
        double u1 = uniform();
        while (u1 <= 1e-300) u1 = uniform();
        const double u2 = uniform();
        const double r = std::sqrt(-2.0 * dlog(u1));
        spare = r * dsin(2.0 * kPi * u2);
        has_spare = true;
        return r * dcos(2.0 * kPi * u2);
    }
};

Vec3 sub(const Vec3& a, const Vec3& b) { return {a[0] - b[0], a[1] - b[1], a[2] - b[2]}; }
Vec3 add(const Vec3& a, const Vec3& b) { return {a[0] + b[0], a[1] + b[1], a[2] + b[2]}; }
Vec3 scale(const Vec3& a, double s) { return {a[0] * s, a[1] * s, a[2] * s}; }
double dot(const Vec3& a, const Vec3& b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
Vec3 cross(const Vec3& a, const Vec3& b) {
    return {a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]};
}
Vec3 normalize(const Vec3& a) { return scale(a, 1.0 / std::sqrt(dot(a, a))); }

Mat3 matmul(const Mat3& a, const Mat3& b) {
    Mat3 c{};
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
            c[i * 3 + j] = a[i * 3 + 0] * b[0 * 3 + j] + a[i * 3 + 1] * b[1 * 3 + j] +
                           a[i * 3 + 2] * b[2 * 3 + j];
    return c;
}
Vec3 matvec(const Mat3& a, const Vec3& v) {
    return {a[0] * v[0] + a[1] * v[1] + a[2] * v[2], a[3] * v[0] + a[4] * v[1] + a[5] * v[2],
            a[6] * v[0] + a[7] * v[1] + a[8] * v[2]};
}
Mat3 transpose(const Mat3& a) { return {a[0], a[3], a[6], a[1], a[4], a[7], a[2], a[5], a[8]}; }

// Rotation by axis-angle vector w (Rodrigues' formula).
Mat3 expso3(const Vec3& w) {
    const double th = std::sqrt(dot(w, w));
    if (th < 1e-15) return {1, 0, 0, 0, 1, 0, 0, 0, 1};
    const Vec3 k = scale(w, 1.0 / th);
    const double c = dcos(th), s = dsin(th), v = 1.0 - c;
    return {c + k[0] * k[0] * v,        k[0] * k[1] * v - k[2] * s, k[0] * k[2] * v + k[1] * s,
            k[1] * k[0] * v + k[2] * s, c + k[1] * k[1] * v,        k[1] * k[2] * v - k[0] * s,
            k[2] * k[0] * v - k[1] * s, k[2] * k[1] * v + k[0] * s, c + k[2] * k[2] * v};
}

struct Pose {  // T_cw
    Mat3 R;
    Vec3 t;
};

// Camera at centre c with optical axis f and world "up" hint: x = f x up, y = f x x (down).
Pose look_along(const Vec3& c, const Vec3& forward, const Vec3& up_hint) {
    const Vec3 z = normalize(forward);
    Vec3 x = cross(z, up_hint);
    if (dot(x, x) < 1e-12) x = cross(z, Vec3{1, 0, 0});
    x = normalize(x);
    const Vec3 y = cross(z, x);
    const Mat3 Rwc = {x[0], y[0], z[0], x[1], y[1], z[1], x[2], y[2], z[2]};
    Pose p;
    p.R = transpose(Rwc);
    p.t = scale(matvec(p.R, c), -1.0);
    return p;
}

struct Intr {
    double k1 = 0.0, k2 = 0.0;
};

// Project; false when behind the camera (Z <= zmin) or outside the image.
bool project(const Pose& p, const Vec3& X, const Intr& in, double zmin, double zmax, double* uv) {
    const Vec3 Xc = add(matvec(p.R, X), p.t);
    if (!(Xc[2] > zmin) || Xc[2] > zmax) return false;
    const double x = Xc[0] / Xc[2], y = Xc[1] / Xc[2];
    const double r2 = x * x + y * y;
    const double d = 1.0 + in.k1 * r2 + in.k2 * r2 * r2;
    uv[0] = kFx * d * x + kCx;
    uv[1] = kFy * d * y + kCy;
    return uv[0] >= 0.0 && uv[0] < kWidth && uv[1] >= 0.0 && uv[1] < kHeight;
}

struct Window {
    std::vector<Pose> cams;
    std::vector<uint8_t> cam_fixed;
    std::vector<Vec3> pts;
    // observations, point-major
    std::vector<int32_t> obs_cam, obs_pt;
};

}  // namespace

struct nav_synth {
    int32_t model = 0;
    std::vector<double> cam_pose, cam_pose_true, pts, pts_true, obs_uv;
    std::vector<uint8_t> cam_fixed, pt_fixed;
    std::vector<int32_t> obs_cam, obs_pt;
    std::vector<int64_t> win_cam, win_pt, win_obs;
    double intr[8] = {kFx, kFy, kCx, kCy, 0, 0, 0, 0};
    double intr_init[8] = {kFx, kFy, kCx, kCy, 0, 0, 0, 0};
};

namespace {

struct Defaults {
    double noise, outliers;
};

// Observe point X from a subset of the visible cameras: all of them when pick <= 0, else a
// random subset of min(pick, visible) cameras, kept in ascending camera order.
int choose_views(Rng& rng, const std::vector<int>& visible, int pick, std::vector<int>& out) {
    out = visible;
    if (pick > 0 && (int)out.size() > pick) {
        for (int i = 0; i < pick; ++i) {
            const int j = i + (int)(rng.uniform() * (double)(out.size() - i)) % (int)(out.size() - i);
            std::swap(out[i], out[j]);
        }
        out.resize(pick);
        std::sort(out.begin(), out.end());
    }
    return (int)out.size();
}

void emit_window(nav_synth* S, Rng& rng, const Window& w, const Intr& truth, double noise,
                 double outliers, double rot_p, double trans_p, double pt_p) {
    const int32_t nc = (int32_t)w.cams.size();
    const int32_t np = (int32_t)w.pts.size();
    S->win_cam.push_back(S->win_cam.back() + nc);
    S->win_pt.push_back(S->win_pt.back() + np);
    S->win_obs.push_back(S->win_obs.back() + (int64_t)w.obs_cam.size());
    for (int32_t c = 0; c < nc; ++c) {
        const Pose& p = w.cams[c];
        Pose q = p;
        if (!w.cam_fixed[c]) {
            // orientation perturbed by exp(om) and the camera centre C = -R^T t by a translation
            // (perturbing t directly would also move the centre by |t| * |om|, metres on a 2 km path)
            const Vec3 om = {rng.normal() * rot_p, rng.normal() * rot_p, rng.normal() * rot_p};
            const Vec3 dC = {rng.normal() * trans_p, rng.normal() * trans_p, rng.normal() * trans_p};
            const Vec3 C = add(scale(matvec(transpose(p.R), p.t), -1.0), dC);
            q.R = matmul(expso3(om), p.R);
            q.t = scale(matvec(q.R, C), -1.0);
        }
        for (int r = 0; r < 3; ++r) {
            for (int k = 0; k < 3; ++k) {
                S->cam_pose_true.push_back(p.R[r * 3 + k]);
                S->cam_pose.push_back(q.R[r * 3 + k]);
            }
            S->cam_pose_true.push_back(p.t[r]);
            S->cam_pose.push_back(q.t[r]);
        }
        S->cam_fixed.push_back(w.cam_fixed[c]);
    }
    for (int32_t i = 0; i < np; ++i) {
        for (int k = 0; k < 3; ++k) {
            S->pts_true.push_back(w.pts[i][k]);
            S->pts.push_back(w.pts[i][k] + rng.normal() * pt_p);
        }
        S->pt_fixed.push_back(0);
    }
    for (size_t o = 0; o < w.obs_cam.size(); ++o) {
        double uv[2];
        project(w.cams[w.obs_cam[o]], w.pts[w.obs_pt[o]], truth, -1e300, 1e300, uv);
        if (outliers > 0.0 && rng.uniform() < outliers) {
            uv[0] = rng.uniform(0.0, kWidth);
            uv[1] = rng.uniform(0.0, kHeight);
        } else {
            uv[0] += rng.normal() * noise;
            uv[1] += rng.normal() * noise;
        }
        S->obs_uv.push_back(uv[0]);
        S->obs_uv.push_back(uv[1]);
        S->obs_cam.push_back(w.obs_cam[o]);
        S->obs_pt.push_back(w.obs_pt[o]);
    }
}

// Generic point sampler: draw points from `sample`, keep those seen by at least `min_views`
// cameras, observe each from `pick()` of them.
template <class SampleFn, class PickFn, class CandFn>
void fill_points(Window& w, Rng& rng, int n_points, const Intr& truth, double zmin, double zmax,
                 int min_views, SampleFn sample, PickFn pick, CandFn candidates) {
    std::vector<int> vis, chosen, cand;
    for (int i = 0; i < n_points; ++i) {
        Vec3 X{};
        int tries = 0;
        for (;;) {
            X = sample();
            vis.clear();
            candidates(X, cand);
            for (int c : cand) {
                double uv[2];
                if (project(w.cams[c], X, truth, zmin, zmax, uv)) vis.push_back(c);
            }
            std::sort(vis.begin(), vis.end());
            if ((int)vis.size() >= min_views || ++tries > 200) break;
        }
        if ((int)vis.size() < 2) continue;  // unobservable after many draws: drop it
        choose_views(rng, vis, pick(), chosen);
        const int32_t pid = (int32_t)w.pts.size();
        w.pts.push_back(X);
        for (int c : chosen) {
            w.obs_cam.push_back(c);
            w.obs_pt.push_back(pid);
        }
    }
}

void all_candidates(const Window& w, std::vector<int>& cand) {
    cand.resize(w.cams.size());
    for (size_t c = 0; c < w.cams.size(); ++c) cand[c] = (int)c;
}

}  // namespace

extern "C" nav_synth* nav_synth_create(const nav_synth_params* prm) {
    if (!prm || prm->family < 0 || prm->family > 4) return nullptr;
    nav_synth* S = new nav_synth();
    S->win_cam.push_back(0);
    S->win_pt.push_back(0);
    S->win_obs.push_back(0);
    Rng rng(prm->seed);
    const int fam = prm->family;
    const Defaults dflt[5] = {{1.0, 0.0}, {1.0, 0.0}, {0.8, 0.0}, {1.0, 0.0}, {1.0, 0.05}};
    const double noise = prm->pixel_noise >= 0 ? prm->pixel_noise : dflt[fam].noise;
    const double outl = prm->outlier_frac >= 0 ? prm->outlier_frac : dflt[fam].outliers;
    const double rot_p = prm->rot_perturb >= 0 ? prm->rot_perturb : 0.01;
    const double trans_p = prm->trans_perturb >= 0 ? prm->trans_perturb : 0.05;
    const double pt_p = prm->point_perturb >= 0 ? prm->point_perturb : 0.05;
    Intr truth;
    const Vec3 up = {0, 0, 1};

    if (fam == 0) {
        // Ring: cameras evenly on a radius-5 m circle at height 0, looking at the origin;
        // points uniform in [-1,1]^3; every camera that images a point observes it.
        Window w;
        const int nc = prm->n_cams > 0 ? prm->n_cams : 10;
        const int np = prm->n_points > 0 ? prm->n_points : 500;
        for (int c = 0; c < nc; ++c) {
            const double a = 2.0 * kPi * c / nc;
            const Vec3 C = {5.0 * dcos(a), 5.0 * dsin(a), 0.0};
            w.cams.push_back(look_along(C, scale(C, -1.0), up));
            w.cam_fixed.push_back(c == 0);
        }
        fill_points(
            w, rng, np, truth, 1e-6, 1e300, 2,
            [&] { return Vec3{rng.uniform(-1, 1), rng.uniform(-1, 1), rng.uniform(-1, 1)}; },
            [] { return 0; }, [&](const Vec3&, std::vector<int>& c) { all_candidates(w, c); });
        emit_window(S, rng, w, truth, noise, outl, rot_p, trans_p, pt_p);
    } else if (fam == 1) {
        // Grid: nx x ny cameras 2 m apart at height 3 m facing down with +-0.1 rad random
        // tilt; points uniform over the ground patch under the grid, height U(0, 2) m.
        Window w;
        const int n_req = prm->n_cams > 0 ? prm->n_cams : 200;
        int ny = std::max(1, (int)std::lround(std::sqrt(n_req / 2.0)));
        int nx = std::max(1, n_req / ny);
        const int np = prm->n_points > 0 ? prm->n_points : 50000;
        const Mat3 Rwc_down = {1, 0, 0, 0, -1, 0, 0, 0, -1};
        for (int j = 0; j < ny; ++j) {
            for (int i = 0; i < nx; ++i) {
                const Vec3 C = {-(nx - 1) + 2.0 * i, -(ny - 1) + 2.0 * j, 3.0};
                const Vec3 tilt = {rng.uniform(-0.1, 0.1), rng.uniform(-0.1, 0.1), 0.0};
                const Mat3 Rwc = matmul(Rwc_down, expso3(tilt));
                Pose p;
                p.R = transpose(Rwc);
                p.t = scale(matvec(p.R, C), -1.0);
                w.cams.push_back(p);
                w.cam_fixed.push_back(w.cams.size() == 1);
            }
        }
        // candidate cameras: the grid cells within 3 cells of the point
        auto cands = [&](const Vec3& X, std::vector<int>& c) {
            c.clear();
            const int ci = (int)std::floor((X[0] + nx) / 2.0), cj = (int)std::floor((X[1] + ny) / 2.0);
            for (int j = std::max(0, cj - 3); j <= std::min(ny - 1, cj + 3); ++j)
                for (int i = std::max(0, ci - 3); i <= std::min(nx - 1, ci + 3); ++i)
                    c.push_back(j * nx + i);
        };
        fill_points(
            w, rng, np, truth, 0.1, 1e300, 2,
            [&] {
                return Vec3{rng.uniform(-(double)nx, (double)nx), rng.uniform(-(double)ny, (double)ny),
                            rng.uniform(0.0, 2.0)};
            },
            [] { return 0; }, cands);
        emit_window(S, rng, w, truth, noise, outl, rot_p, trans_p, pt_p);
    } else if (fam == 2) {
        // Windows: keyframes U{min..max} on a smooth random trajectory (0.3 m, 0.05 rad steps),
        // points U{min..max} uniform in a 4 m box ahead; 3-8 views per point; the first two
        // keyframes of each window are fixed.
        const int nwin = prm->n_windows > 0 ? prm->n_windows : 512;
        const int kmax = prm->n_cams > 0 ? prm->n_cams : 20;
        const int kmin = prm->min_cams > 0 ? std::min(prm->min_cams, kmax) : std::min(5, kmax);
        const int pmax = prm->n_points > 0 ? prm->n_points : 3000;
        const int pmin = prm->min_points > 0 ? std::min(prm->min_points, pmax) : std::min(200, pmax);
        for (int wi = 0; wi < nwin; ++wi) {
            Window w;
            const int nc = rng.uniform_int(kmin, kmax);
            const int np = rng.uniform_int(pmin, pmax);
            Mat3 Rwc = {1, 0, 0, 0, 1, 0, 0, 0, 1};
            Vec3 C = {0, 0, 0};
            Vec3 omega = {0, 0, 0};
            Vec3 zsum = {0, 0, 0}, csum = {0, 0, 0};
            for (int c = 0; c < nc; ++c) {
                Pose p;
                p.R = transpose(Rwc);
                p.t = scale(matvec(p.R, C), -1.0);
                w.cams.push_back(p);
                w.cam_fixed.push_back(c < 2);
                zsum = add(zsum, Vec3{Rwc[2], Rwc[5], Rwc[8]});
                csum = add(csum, C);
                // smooth heading change of 0.05 rad per step
                const Vec3 n = {rng.normal(), rng.normal(), rng.normal()};
                omega = add(scale(omega, 0.7), scale(n, 0.3));
                const Vec3 om = scale(normalize(omega), 0.05);
                Rwc = matmul(Rwc, expso3(om));
                const Vec3 xc = {Rwc[0], Rwc[3], Rwc[6]}, yc = {Rwc[1], Rwc[4], Rwc[7]},
                           zc = {Rwc[2], Rwc[5], Rwc[8]};
                // draws sequenced explicitly: function arguments have no evaluation order
                const double jz = rng.normal();
                const double jy = rng.normal();
                const Vec3 d = normalize(add(xc, add(scale(zc, 0.3 * jz), scale(yc, 0.3 * jy))));
                C = add(C, scale(d, 0.3));
            }
            const Vec3 box_c = add(scale(csum, 1.0 / nc), scale(normalize(zsum), 6.0));
            fill_points(
                w, rng, np, truth, 0.1, 1e300, 3,
                [&] {
                    return add(box_c, Vec3{rng.uniform(-2, 2), rng.uniform(-2, 2), rng.uniform(-2, 2)});
                },
                [&] { return rng.uniform_int(3, 8); },
                [&](const Vec3&, std::vector<int>& c) { all_candidates(w, c); });
            emit_window(S, rng, w, truth, noise, outl, rot_p, trans_p, pt_p);
        }
    } else if (fam == 3) {
        // Cap: cameras on a radius-6 m sphere cap (polar angle <= 60 deg, Fibonacci spiral)
        // looking at the centre; points in [-2,2]^3; about 6 (U{4..8}) views per point.
        Window w;
        const int nc = prm->n_cams > 0 ? prm->n_cams : 50;
        const int np = prm->n_points > 0 ? prm->n_points : 10000;
        const double golden = kPi * (3.0 - std::sqrt(5.0));
        const double cos_min = dcos(60.0 * kPi / 180.0);
        for (int c = 0; c < nc; ++c) {
            const double z = 1.0 - (1.0 - cos_min) * (c + 0.5) / nc;
            const double r = std::sqrt(std::max(0.0, 1.0 - z * z));
            const double a = golden * c;
            const Vec3 C = {6.0 * r * dcos(a), 6.0 * r * dsin(a), 6.0 * z};
            w.cams.push_back(look_along(C, scale(C, -1.0), Vec3{0, 1, 0}));
            w.cam_fixed.push_back(c == 0);
        }
        fill_points(
            w, rng, np, truth, 0.1, 1e300, 2,
            [&] { return Vec3{rng.uniform(-2, 2), rng.uniform(-2, 2), rng.uniform(-2, 2)}; },
            [&] { return rng.uniform_int(4, 8); },
            [&](const Vec3&, std::vector<int>& c) { all_candidates(w, c); });
        emit_window(S, rng, w, truth, noise, outl, rot_p, trans_p, pt_p);
    } else {
        // Figure-eight: cameras 1.5 m above a three-loop lemniscate (x = A sin s,
        // y = B sin s cos s) scaled to 2000 m in total, facing along the path with 0.05 rad
        // yaw jitter; points in a 10 m band around the path, height U(0, 3) m; U{6..10}
        // views per point (depth 1-40 m); radial k1 = -0.1, k2 = 0.01; 5% outliers.
        S->model = 1;
        truth.k1 = -0.1;
        truth.k2 = 0.01;
        Window w;
        const int nc = prm->n_cams > 0 ? prm->n_cams : 1000;
        const int np = prm->n_points > 0 ? prm->n_points : 500000;
        const double total_len = 2000.0 * nc / 1000.0;
        const int loops = 3;
        // arc-length table of the base curve
        const int nt = 20000;
        std::vector<double> arc(nt + 1, 0.0);
        auto curve = [](double s) { return Vec3{150.0 * dsin(s), 100.0 * dsin(s) * dcos(s), 0.0}; };
        for (int k = 1; k <= nt; ++k) {
            const Vec3 a = curve(2 * kPi * (k - 1) / nt), b = curve(2 * kPi * k / nt);
            arc[k] = arc[k - 1] + std::sqrt(dot(sub(b, a), sub(b, a)));
        }
        const double sc = (total_len / loops) / arc[nt];
        auto at_arc = [&](double L) {  // parameter s for arc length L on one loop (scaled)
            L = std::fmod(L, arc[nt] * sc);
            if (L < 0) L += arc[nt] * sc;
            const double target = L / sc;
            const int k = (int)(std::upper_bound(arc.begin(), arc.end(), target) - arc.begin()) - 1;
            const int kk = std::min(std::max(k, 0), nt - 1);
            const double f = (target - arc[kk]) / std::max(1e-12, arc[kk + 1] - arc[kk]);
            return 2 * kPi * (kk + f) / nt;
        };
        auto pos = [&](double s, double lateral, double h) {
            const Vec3 p = scale(curve(s), sc);
            const Vec3 d = normalize(sub(curve(s + 1e-4), curve(s - 1e-4)));
            const Vec3 n = {-d[1], d[0], 0.0};
            return add(add(p, scale(n, lateral)), Vec3{0, 0, h});
        };
        const double step = total_len / nc;
        std::vector<Vec3> centres;
        for (int c = 0; c < nc; ++c) {
            const double L = c * step;
            const int loop = (int)(L / (total_len / loops));
            const double s = at_arc(L);
            const Vec3 C = pos(s, 0.6 * (loop - 1), 1.5);
            const Vec3 d = normalize(sub(curve(s + 1e-4), curve(s - 1e-4)));
            const double yaw = rng.normal() * 0.05;
            const Vec3 f = {d[0] * dcos(yaw) - d[1] * dsin(yaw),
                            d[0] * dsin(yaw) + d[1] * dcos(yaw), 0.0};
            w.cams.push_back(look_along(C, f, up));
            w.cam_fixed.push_back(c == 0);
            centres.push_back(C);
        }
        // spatial hash of camera centres (20 m cells) for candidate lookup
        std::unordered_map<int64_t, std::vector<int>> grid;
        auto key = [](int gx, int gy) { return ((int64_t)gx << 32) ^ (int64_t)(uint32_t)gy; };
        for (int c = 0; c < nc; ++c)
            grid[key((int)std::floor(centres[c][0] / 20.0), (int)std::floor(centres[c][1] / 20.0))].push_back(c);
        auto cands = [&](const Vec3& X, std::vector<int>& c) {
            c.clear();
            const int gx = (int)std::floor(X[0] / 20.0), gy = (int)std::floor(X[1] / 20.0);
            for (int dy = -2; dy <= 2; ++dy)
                for (int dx = -2; dx <= 2; ++dx) {
                    auto it = grid.find(key(gx + dx, gy + dy));
                    if (it != grid.end()) c.insert(c.end(), it->second.begin(), it->second.end());
                }
        };
        fill_points(
            w, rng, np, truth, 1.0, 40.0, 2,
            [&] {
                const double L = rng.uniform(0.0, arc[nt] * sc);
                const double lateral = rng.uniform(-5.0, 5.0);
                const double height = rng.uniform(0.0, 3.0);
                return pos(at_arc(L), lateral, height);
            },
            [&] { return rng.uniform_int(6, 10); }, cands);
        emit_window(S, rng, w, truth, noise, outl, rot_p, trans_p, pt_p);
        S->intr_init[4] = -0.08;
        S->intr_init[5] = 0.005;
    }
    S->intr[4] = truth.k1;
    S->intr[5] = truth.k2;
    if (fam != 4) {
        S->intr_init[4] = truth.k1;
        S->intr_init[5] = truth.k2;
    }
    return S;
}

extern "C" void nav_synth_destroy(nav_synth* s) { delete s; }

extern "C" void nav_synth_counts(const nav_synth* s, int64_t* nw, int64_t* nc, int64_t* np,
                                 int64_t* no, int32_t* model) {
    if (nw) *nw = (int64_t)s->win_cam.size() - 1;
    if (nc) *nc = (int64_t)s->cam_fixed.size();
    if (np) *np = (int64_t)s->pt_fixed.size();
    if (no) *no = (int64_t)s->obs_cam.size();
    if (model) *model = s->model;
}

extern "C" int64_t nav_synth_size(const nav_synth* s, int32_t id) {
    switch (id) {
        case NAV_SYNTH_CAM_POSE: return (int64_t)s->cam_pose.size();
        case NAV_SYNTH_CAM_POSE_TRUE: return (int64_t)s->cam_pose_true.size();
        case NAV_SYNTH_CAM_FIXED: return (int64_t)s->cam_fixed.size();
        case NAV_SYNTH_POINTS: return (int64_t)s->pts.size();
        case NAV_SYNTH_POINTS_TRUE: return (int64_t)s->pts_true.size();
        case NAV_SYNTH_POINT_FIXED: return (int64_t)s->pt_fixed.size();
        case NAV_SYNTH_OBS_UV: return (int64_t)s->obs_uv.size();
        case NAV_SYNTH_OBS_CAM: return (int64_t)s->obs_cam.size();
        case NAV_SYNTH_OBS_POINT: return (int64_t)s->obs_pt.size();
        case NAV_SYNTH_WIN_CAM_OFF: return (int64_t)s->win_cam.size();
        case NAV_SYNTH_WIN_POINT_OFF: return (int64_t)s->win_pt.size();
        case NAV_SYNTH_WIN_OBS_OFF: return (int64_t)s->win_obs.size();
        case NAV_SYNTH_INTRINSICS: return 8;
        case NAV_SYNTH_INTRINSICS_INIT: return 8;
        default: return -1;
    }
}

extern "C" int32_t nav_synth_copy(const nav_synth* s, int32_t id, void* dst) {
    if (!s || !dst) return -1;
    auto cp = [&](const auto& v) {
        if (!v.empty()) std::memcpy(dst, v.data(), v.size() * sizeof(v[0]));
        return 0;
    };
    switch (id) {
        case NAV_SYNTH_CAM_POSE: return cp(s->cam_pose);
        case NAV_SYNTH_CAM_POSE_TRUE: return cp(s->cam_pose_true);
        case NAV_SYNTH_CAM_FIXED: return cp(s->cam_fixed);
        case NAV_SYNTH_POINTS: return cp(s->pts);
        case NAV_SYNTH_POINTS_TRUE: return cp(s->pts_true);
        case NAV_SYNTH_POINT_FIXED: return cp(s->pt_fixed);
        case NAV_SYNTH_OBS_UV: return cp(s->obs_uv);
        case NAV_SYNTH_OBS_CAM: return cp(s->obs_cam);
        case NAV_SYNTH_OBS_POINT: return cp(s->obs_pt);
        case NAV_SYNTH_WIN_CAM_OFF: return cp(s->win_cam);
        case NAV_SYNTH_WIN_POINT_OFF: return cp(s->win_pt);
        case NAV_SYNTH_WIN_OBS_OFF: return cp(s->win_obs);
        case NAV_SYNTH_INTRINSICS: std::memcpy(dst, s->intr, sizeof(s->intr)); return 0;
        case NAV_SYNTH_INTRINSICS_INIT: std::memcpy(dst, s->intr_init, sizeof(s->intr_init)); return 0;
        default: return -1;
    }
}
