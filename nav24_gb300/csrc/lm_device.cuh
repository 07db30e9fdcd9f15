// lm_device.cuh - device code shared by the window engine and the grid engine: the argument
// block, the thread-range view, the per-point / per-edge phases of one LM iteration (point-major
// linearization, damped point blocks and A = W L^T, back-substitution) and the robust cost.
// Each phase loops over points p = gt, gt + CT, ... so it runs unchanged over one window (a CTA
// cluster) or over a whole problem (a grid).
#pragma once

#include "engine.hpp"

namespace navba {
namespace {

struct SmemHead;  // the window engine's shared-memory head (window_engine.cu)

template <class Real>
struct WinArgs {
    const WinDesc* win;
    int32_t n_win;
    int32_t n_big;            // window engine: the first n_big windows of `order` are solved by clusters
    const int32_t* order;
    int32_t* queue;           // window engine: [0] the clusters' queue, [1] the single CTAs' queue
    const CamState* cam_init;
    const int32_t* cam_free;
    const double* pt_init;
    const int32_t* pt_free;
    const int32_t* pt_eoff;
    const int32_t* edge_cam;
    const int32_t* edge_fc;   // free index of each edge's camera, or -1
    const int32_t* edge_pt;
    const double* edge_uv;
    Real* edge_uvr;           // window engine, mixed form: edge_uv rounded to Real (null: rounded per use)
    double* x[2];
    Real* xr[2];              // window engine, mixed form: x rounded to Real, kept with x (null: per use)
    Real* pt_vg;
    Real* pt_lt;
    Real* edge_w;             // FP64 form: W_e = w J_c^T J_p per edge; null: recomputed (mixed form)
    Real* edge_a;
    int32_t jfact;            // window engine, mixed form, pinhole: edge_a holds Jacobian-factored
                              // records (JRec) instead of A
    Real* edge_e[2];          // mixed form: residual (u, v) of each edge at the current / trial state
    const Real* edge_ep;      // grid engine, mixed form: each edge's residual at the linearization
                              // state, evaluated in FP64 by the cost pass (null: evaluated in Real)
    int32_t* cam_list;
    double* s_glob;           // window engine, mixed form: the windows' FP64 reduced systems (WinDesc::s0)
    uint32_t* pairs;
    CamState* cam_out;
    double* pt_out;
    double* trace;
    int32_t trace_stride;
    WinStats* stats;
    double* debug;
    double debug_lambda;
    Intr intr;
    LmOptions lm;
    int32_t max_m, max_ncam;
    unsigned long long* phase;  // optional per-phase SM-cycle totals (rank 0 view), or null
};

NAVBA_HD int tri(int r, int c) { return r * (r + 1) / 2 + c; }  // packed lower index, c <= r

// Per-CTA view of the cluster working on a window.
struct CC {
    int rank, csize;
    int gt, CT;   // thread index / count over the cluster
    int gw, CW;   // warp index / count over the cluster
    int lane, wid, nw;
    SmemHead* s;   // this CTA's head
    SmemHead* s0;  // rank 0's head (distributed shared memory)
    double* S0;    // the reduced system (rank 0's shared memory, or the mixed form's global scratch)
    float* S0f;    // mixed form: rank 0's FP32 copy of it (factored in place), else null
    double* bs0;   // rank 0's right-hand side / step
};

template <class Real>
__device__ __forceinline__ void cam_real(const CamState& c, Real* o) {
#pragma unroll
    for (int k = 0; k < 9; ++k) o[k] = (Real)c.R[k];
    o[9] = (Real)c.t[0];
    o[10] = (Real)c.t[1];
    o[11] = (Real)c.t[2];
}

// Per-edge 18-value records (W, A) and per-point 12-value records (V|g, L|t), moved with
// 16-byte vector accesses: FP32 records are padded to 20 floats (80 B), FP64 ones are 144 B.
template <class Real>
struct Rec;

template <>
struct Rec<float> {
    static constexpr int kEdge = 20;
    static __device__ __forceinline__ void load18(const float* p, float* v) {
        const float4* q = reinterpret_cast<const float4*>(p);
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const float4 t = q[k];
            v[4 * k] = t.x; v[4 * k + 1] = t.y; v[4 * k + 2] = t.z; v[4 * k + 3] = t.w;
        }
        const float2 t = reinterpret_cast<const float2*>(p)[8];
        v[16] = t.x;
        v[17] = t.y;
    }
    static __device__ __forceinline__ void store18(float* p, const float* v) {
        float4* q = reinterpret_cast<float4*>(p);
#pragma unroll
        for (int k = 0; k < 4; ++k) q[k] = make_float4(v[4 * k], v[4 * k + 1], v[4 * k + 2], v[4 * k + 3]);
        reinterpret_cast<float2*>(p)[8] = make_float2(v[16], v[17]);
    }
    static __device__ __forceinline__ void load12(const float* p, float* v) {
        const float4* q = reinterpret_cast<const float4*>(p);
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const float4 t = q[k];
            v[4 * k] = t.x; v[4 * k + 1] = t.y; v[4 * k + 2] = t.z; v[4 * k + 3] = t.w;
        }
    }
    static __device__ __forceinline__ void store12(float* p, const float* v) {
        float4* q = reinterpret_cast<float4*>(p);
#pragma unroll
        for (int k = 0; k < 3; ++k) q[k] = make_float4(v[4 * k], v[4 * k + 1], v[4 * k + 2], v[4 * k + 3]);
    }
};

template <>
struct Rec<double> {
    static constexpr int kEdge = 18;
    static __device__ __forceinline__ void load18(const double* p, double* v) {
        const double2* q = reinterpret_cast<const double2*>(p);
#pragma unroll
        for (int k = 0; k < 9; ++k) {
            const double2 t = q[k];
            v[2 * k] = t.x;
            v[2 * k + 1] = t.y;
        }
    }
    static __device__ __forceinline__ void store18(double* p, const double* v) {
        double2* q = reinterpret_cast<double2*>(p);
#pragma unroll
        for (int k = 0; k < 9; ++k) q[k] = make_double2(v[2 * k], v[2 * k + 1]);
    }
    static __device__ __forceinline__ void load12(const double* p, double* v) {
        const double2* q = reinterpret_cast<const double2*>(p);
#pragma unroll
        for (int k = 0; k < 6; ++k) {
            const double2 t = q[k];
            v[2 * k] = t.x;
            v[2 * k + 1] = t.y;
        }
    }
    static __device__ __forceinline__ void store12(double* p, const double* v) {
        double2* q = reinterpret_cast<double2*>(p);
#pragma unroll
        for (int k = 0; k < 6; ++k) q[k] = make_double2(v[2 * k], v[2 * k + 1]);
    }
};

// Point gp's state and edge e's observation in Real, from the Real copies where they are kept
// (XR, A.edge_uvr), else rounded from FP64 here: both give the same values.
template <class Real>
__device__ __forceinline__ void point_real(const double* X, const Real* XR, long long gp, Real* o) {
    if constexpr (sizeof(Real) == 4) {
        if (XR) {
            const float4 t = *reinterpret_cast<const float4*>(XR + 4 * gp);
            o[0] = t.x;
            o[1] = t.y;
            o[2] = t.z;
            return;
        }
    }
    o[0] = (Real)X[4 * gp];
    o[1] = (Real)X[4 * gp + 1];
    o[2] = (Real)X[4 * gp + 2];
}

template <class Real>
__device__ __forceinline__ void obs_real(const WinArgs<Real>& A, long long e, Real* z) {
    if constexpr (sizeof(Real) == 4) {
        if (A.edge_uvr) {
            const float2 t = *reinterpret_cast<const float2*>(A.edge_uvr + 2 * e);
            z[0] = t.x;
            z[1] = t.y;
            return;
        }
    }
    z[0] = (Real)A.edge_uv[2 * e];
    z[1] = (Real)A.edge_uv[2 * e + 1];
}

// Trial point gp = X + d: the FP64 state, and its Real copy where one is kept.
template <class Real>
__device__ __forceinline__ void store_trial_point(const double* Xc, double* Xt, Real* XRt, long long gp, Real d0,
                                                  Real d1, Real d2) {
    const double x0 = Xc[4 * gp + 0] + (double)d0, x1 = Xc[4 * gp + 1] + (double)d1, x2 = Xc[4 * gp + 2] + (double)d2;
    Xt[4 * gp + 0] = x0;
    Xt[4 * gp + 1] = x1;
    Xt[4 * gp + 2] = x2;
    if constexpr (sizeof(Real) == 4) {
        if (XRt) *reinterpret_cast<float4*>(XRt + 4 * gp) = make_float4((float)x0, (float)x1, (float)x2, 0.f);
    }
}

// Jacobian-factored edge record (mixed form, pinhole model), 12 floats: u = x / z, v = y / z,
// iz = 1 / z of the point in the camera at the linearization state, B = w J_p L^T (2x3, row-major)
// and the point's t = L g.  A = W L^T = w J_c^T J_p L^T = J_c^T B, and J_c follows from (u, v, iz)
// (pinhole_jc), so the record carries A in 48 bytes instead of 80: A_i A_j^T = J_ci^T (B_i B_j^T)
// J_cj and A^T d = B^T (J_c d).
struct JRec {
    static constexpr int kEdge = 12;
    static __device__ __forceinline__ void load(const float* p, float* v) { Rec<float>::load12(p, v); }
};

// u -= A_e^T d = B^T (J_c d) from a Jacobian-factored record and the edge camera's step d.
template <class Real, class DC>
__device__ __forceinline__ void sub_at_d_rec(const Real* rec, const DC* d, Real fx, Real fy, Real& u0, Real& u1,
                                             Real& u2) {
    Real jc[12];
    pinhole_jc(fx, fy, rec[0], rec[1], rec[2], jc);
    Real j0 = Real(0), j1 = Real(0);
#pragma unroll
    for (int r = 0; r < 6; ++r) {
        const Real dr = (Real)d[r];
        j0 += jc[r] * dr;
        j1 += jc[6 + r] * dr;
    }
    u0 -= rec[3] * j0 + rec[6] * j1;
    u1 -= rec[4] * j0 + rec[7] * j1;
    u2 -= rec[5] * j0 + rec[8] * j1;
}

// u -= A_e^T d for edge e and its camera's step d (6 values).
template <class Real, class DC>
__device__ __forceinline__ void sub_at_d(const WinArgs<Real>& A, long long e, const DC* d, Real fx, Real fy, Real& u0,
                                         Real& u1, Real& u2) {
    if constexpr (sizeof(Real) == 4) {
        if (A.jfact) {
            Real rec[12];
            JRec::load(A.edge_a + (long long)JRec::kEdge * e, rec);
            sub_at_d_rec(rec, d, fx, fy, u0, u1, u2);
            return;
        }
    }
    Real Ae[18];
    Rec<Real>::load18(A.edge_a + (long long)Rec<Real>::kEdge * e, Ae);
#pragma unroll
    for (int r = 0; r < 6; ++r) {
        const Real dr = (Real)d[r];
        u0 -= Ae[r * 3 + 0] * dr;
        u1 -= Ae[r * 3 + 1] * dr;
        u2 -= Ae[r * 3 + 2] * dr;
    }
}

// The 12 values (R row-major, t) of camera record cr into registers with 16-byte loads (camera
// records start 16-byte aligned): three loads in FP32 instead of twelve.
template <class Real>
__device__ __forceinline__ void cam_load(const Real* cr, Real* o) {
    if constexpr (sizeof(Real) == 4) {
        const float4* q = reinterpret_cast<const float4*>(cr);
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const float4 t = q[k];
            o[4 * k] = t.x; o[4 * k + 1] = t.y; o[4 * k + 2] = t.z; o[4 * k + 3] = t.w;
        }
    } else {
        const double2* q = reinterpret_cast<const double2*>(cr);
#pragma unroll
        for (int k = 0; k < 6; ++k) {
            const double2 t = q[k];
            o[2 * k] = t.x;
            o[2 * k + 1] = t.y;
        }
    }
}

// Warp reduce-scatter of 36 per-lane values (a 6x6 block's partial sums): each exchange sends the
// half of the lane's current values that its partner keeps, so 32 + 16 + 8 + 4 + 2 = 62 shuffles
// instead of 36 x 5 for a full butterfly.  Lane l ends with the sums of entries rs36_slot(l) and
// rs36_slot(l) + 1 (entries 36..63 are zero padding).  v is clobbered.
__device__ __forceinline__ int rs36_slot(int lane) {
    return 32 * ((lane >> 4) & 1) + 16 * ((lane >> 3) & 1) + 8 * ((lane >> 2) & 1) + 4 * ((lane >> 1) & 1) + 2 * (lane & 1);
}

template <class T>
__device__ __forceinline__ void reduce_scatter36(T* v, int lane, T& s0, T& s1) {
    constexpr unsigned kAll = 0xffffffffu;
    {
        const bool hi = (lane & 16) != 0;
#pragma unroll
        for (int i = 0; i < 32; ++i) {
            const T a = v[i], b = i + 32 < 36 ? v[i + 32 < 36 ? i + 32 : 0] : T(0);
            const T send = hi ? a : b, keep = hi ? b : a;
            v[i] = keep + __shfl_xor_sync(kAll, send, 16);
        }
    }
#pragma unroll
    for (int st = 0; st < 4; ++st) {
        const int o = 8 >> st, n = 16 >> st;
        const bool hi = (lane & o) != 0;
#pragma unroll
        for (int i = 0; i < n; ++i) {
            const T send = hi ? v[i] : v[i + n], keep = hi ? v[i + n] : v[i];
            v[i] = keep + __shfl_xor_sync(kAll, send, o);
        }
    }
    s0 = v[0];
    s1 = v[1];
}

// v[k] for a runtime k < N (0 otherwise) from a register array, by selects (no local-memory copy).
template <int N, class Real>
__device__ __forceinline__ Real lane_value(const Real* v, int k) {
    Real o = Real(0);
#pragma unroll
    for (int x = 0; x < N; ++x)
        if (x == k) o = v[x];
    return o;
}

// edge_linearize for edge e.  With A.edge_ep (the grid engine's mixed form) the residual and the
// robust weight come from the edge's residual stored by the FP64 cost pass of the same state: in
// FP32, R X + t of world coordinates of ~100 m keeps ~1e-5 m, which moves the residuals by up to
// 1e-2 px and alike for all edges of a camera (its translation's rounding); the gradient built from
// such residuals stalls the LM near convergence.  The Jacobians keep the Real evaluation.
template <class Real>
__device__ __forceinline__ void edge_linearize_e(const WinArgs<Real>& A, long long e, const Real* cr, const Real* Xr,
                                                 const Real* z, Real delta, EdgeLin<Real>& L) {
    edge_linearize<Real>(A.intr, cr, cr + 9, Xr, z, A.lm.robust != 0, delta, L);
    if constexpr (sizeof(Real) == 4) {
        if (A.edge_ep) {
            const float2 ep = reinterpret_cast<const float2*>(A.edge_ep)[e];
            L.e[0] = ep.x;
            L.e[1] = ep.y;
            huber<Real>(ep.x * ep.x + ep.y * ep.y, A.lm.robust != 0, delta, L.rho, L.w);
        }
    }
}

// Cluster-split robust chi2 of the window for cameras `camc` (12 values per camera, precision
// Cost) and points X; returns this thread's partial sum.  e_out != null: each edge's residual is
// also written there (2 values per edge, rounded to Real).
template <class Cost, class Real>
__device__ double cost_partial(const WinArgs<Real>& A, const CC& c, const WinDesc& D, const Cost* camc,
                               const double* X, Real* e_out = nullptr) {
    double acc = 0.0;
    const Cost delta = (Cost)A.lm.huber_delta;
    for (int p = c.gt; p < D.npt; p += c.CT) {
        const int gp = D.pt0 + p;
        const Cost Xr[3] = {(Cost)X[4LL * gp], (Cost)X[4LL * gp + 1], (Cost)X[4LL * gp + 2]};
        const int e1 = A.pt_eoff[gp + 1];
        for (int e = A.pt_eoff[gp]; e < e1; ++e) {
            Cost cr[12];
            cam_load(camc + 12 * A.edge_cam[e], cr);
            const Cost z[2] = {(Cost)A.edge_uv[2LL * e], (Cost)A.edge_uv[2LL * e + 1]};
            if (e_out) {
                Cost Xc[3], uv[2];
                transform(cr, cr + 9, Xr, Xc);
                project<Cost>(A.intr, Xc, uv, nullptr);
                const Cost e0 = z[0] - uv[0], e1v = z[1] - uv[1];
                double rho;
                Cost w;
                huber<Cost>(e0 * e0 + e1v * e1v, A.lm.robust != 0, delta, rho, w);
                acc += rho;
                e_out[2LL * e] = (Real)e0;
                e_out[2LL * e + 1] = (Real)e1v;
            } else {
                acc += edge_cost<Cost>(A.intr, cr, cr + 9, Xr, z, A.lm.robust != 0, delta);
            }
        }
    }
    return acc;
}

// Point-major linearization: V_p, g_p and, when edge_w is set, W_e; returns this thread's max |diag V|.
template <class Real>
__device__ double linearize_points(const WinArgs<Real>& A, const CC& c, const WinDesc& D, const Real* camr,
                                   const double* X, const Real* XR = nullptr) {
    const Real delta = (Real)A.lm.huber_delta;
    double mx = 0.0;
    for (int p = c.gt; p < D.npt; p += c.CT) {
        const int gp = D.pt0 + p;
        if (A.pt_free[gp] < 0) continue;
        Real Xr[3];
        point_real(X, XR, gp, Xr);
        Real V[6] = {0, 0, 0, 0, 0, 0}, g[3] = {0, 0, 0};
        const int e0 = A.pt_eoff[gp], e1 = A.pt_eoff[gp + 1];
        // the next edge's camera and observation are loaded before the current edge's products
        int cam_n = A.edge_cam[e0];
        Real z_n[2];
        obs_real(A, e0, z_n);
        for (int e = e0; e < e1; ++e) {
            const int cam = cam_n;
            const Real z[2] = {z_n[0], z_n[1]};
            if (e + 1 < e1) {
                cam_n = A.edge_cam[e + 1];
                obs_real(A, e + 1, z_n);
            }
            Real cr[12];
            cam_load(camr + 12 * cam, cr);
            EdgeLin<Real> L;
            edge_linearize_e<Real>(A, e, cr, Xr, z, delta, L);
            const Real w = L.w;
            const Real* jp = L.jp;
            V[0] += w * (jp[0] * jp[0] + jp[3] * jp[3]);
            V[1] += w * (jp[0] * jp[1] + jp[3] * jp[4]);
            V[2] += w * (jp[0] * jp[2] + jp[3] * jp[5]);
            V[3] += w * (jp[1] * jp[1] + jp[4] * jp[4]);
            V[4] += w * (jp[1] * jp[2] + jp[4] * jp[5]);
            V[5] += w * (jp[2] * jp[2] + jp[5] * jp[5]);
            const Real we0 = -w * L.e[0], we1 = -w * L.e[1];
            g[0] += jp[0] * we0 + jp[3] * we1;
            g[1] += jp[1] * we0 + jp[4] * we1;
            g[2] += jp[2] * we0 + jp[5] * we1;
            if (A.edge_w && A.edge_fc[e] >= 0) {
                Real W[18];
#pragma unroll
                for (int r = 0; r < 6; ++r)
#pragma unroll
                    for (int k = 0; k < 3; ++k) W[r * 3 + k] = w * (L.jc[r] * jp[k] + L.jc[6 + r] * jp[3 + k]);
                Rec<Real>::store18(A.edge_w + (long long)Rec<Real>::kEdge * e, W);
            }
        }
        const Real vgv[12] = {V[0], V[1], V[2], V[3], V[4], V[5], g[0], g[1], g[2], Real(0), Real(0), Real(0)};
        Rec<Real>::store12(A.pt_vg + 12LL * gp, vgv);
        mx = fmax(mx, (double)fmax(fabs(V[0]), fmax(fabs(V[3]), fabs(V[5]))));
    }
    return mx;
}

// Point gp's damped block: R R^T = V + lambda I, L = R^-1 (packed lower: l00 l10 l11 l20 l21 l22),
// t = L g; ltv = (L, t, 0 0 0) is also stored in pt_lt.  Returns false if V + lambda I is not
// positive definite.
template <class Real>
__device__ __forceinline__ bool point_factor(const WinArgs<Real>& A, long long gp, Real lam, Real* ltv) {
    Real vg[12];
    Rec<Real>::load12(A.pt_vg + 12LL * gp, vg);
    const Real v00 = vg[0] + lam, v01 = vg[1], v02 = vg[2], v11 = vg[3] + lam, v12 = vg[4], v22 = vg[5] + lam;
    const Real r00 = sqrt(v00);
    const Real r10 = v01 / r00, r20 = v02 / r00;
    const Real d11 = v11 - r10 * r10;
    const Real r11 = sqrt(d11);
    const Real r21 = (v12 - r20 * r10) / r11;
    const Real d22 = v22 - r20 * r20 - r21 * r21;
    const Real r22 = sqrt(d22);
    const Real l00 = Real(1) / r00, l11 = Real(1) / r11, l22 = Real(1) / r22;
    const Real l10 = -r10 * l00 * l11;
    const Real l21 = -r21 * l11 * l22;
    const Real l20 = -(r20 * l00 + r21 * l10) * l22;
    ltv[0] = l00; ltv[1] = l10; ltv[2] = l11; ltv[3] = l20; ltv[4] = l21; ltv[5] = l22;
    ltv[6] = l00 * vg[6];
    ltv[7] = l10 * vg[6] + l11 * vg[7];
    ltv[8] = l20 * vg[6] + l21 * vg[7] + l22 * vg[8];
    ltv[9] = ltv[10] = ltv[11] = Real(0);
    Rec<Real>::store12(A.pt_lt + 12LL * gp, ltv);
    return v00 > Real(0) && d11 > Real(0) && d22 > Real(0);
}

// Jacobian-factored record of edge e (free camera, free point) from the point's ltv (point_factor),
// its camera cr and observation z, at the linearization state (cr, Xr).
template <class Real>
__device__ __forceinline__ void edge_jrec(const WinArgs<Real>& A, long long e, const Real* cr, const Real* z,
                                          const Real* Xr, const Real* ltv, Real delta) {
    EdgeLin<Real> L;
    edge_linearize<Real>(A.intr, cr, cr + 9, Xr, z, A.lm.robust != 0, delta, L);
    const Real iz = Real(1) / L.xc[2];
    Real rec[12];
    rec[0] = L.xc[0] * iz;
    rec[1] = L.xc[1] * iz;
    rec[2] = iz;
#pragma unroll
    for (int s2 = 0; s2 < 2; ++s2) {
        const Real j0 = L.w * L.jp[s2 * 3 + 0], j1 = L.w * L.jp[s2 * 3 + 1], j2 = L.w * L.jp[s2 * 3 + 2];
        rec[3 + s2 * 3 + 0] = j0 * ltv[0];
        rec[3 + s2 * 3 + 1] = j0 * ltv[1] + j1 * ltv[2];
        rec[3 + s2 * 3 + 2] = j0 * ltv[3] + j1 * ltv[4] + j2 * ltv[5];
    }
    rec[9] = ltv[6];
    rec[10] = ltv[7];
    rec[11] = ltv[8];
    Rec<Real>::store12(A.edge_a + (long long)JRec::kEdge * e, rec);
}

// Per free point: R R^T = V + lambda I, L = R^-1, t = L g, A_e = W_e L^T.  W_e = w J_c^T J_p is read
// from edge_w (FP64 form, where recomputing costs FP64-pipe time) or recomputed from the edge's
// Jacobians at the current state (mixed form: camr, X are the state the point blocks were
// linearized at, the same arithmetic gives the same W, and no per-edge record round-trips through
// memory).  Returns the number of points whose damped block was not positive definite.
template <class Real>
__device__ int schur_points(const WinArgs<Real>& A, const CC& c, const WinDesc& D, double lambda, const Real* camr,
                            const double* X, const Real* XR = nullptr) {
    const Real lam = (Real)lambda;
    const Real delta = (Real)A.lm.huber_delta;
    int bad = 0;
    for (int p = c.gt; p < D.npt; p += c.CT) {
        const int gp = D.pt0 + p;
        if (A.pt_free[gp] < 0) continue;
        Real ltv[12];
        bad += point_factor(A, gp, lam, ltv) ? 0 : 1;
        const Real l00 = ltv[0], l10 = ltv[1], l11 = ltv[2], l20 = ltv[3], l21 = ltv[4], l22 = ltv[5];
        Real Xr[3];
        point_real(X, XR, gp, Xr);
        const int e1 = A.pt_eoff[gp + 1];
        if constexpr (sizeof(Real) == 4) {
            if (A.jfact) {
                // Jacobian-factored records; the next edge's camera, observation and free index are
                // loaded before the current edge's record is formed
                const int e0 = A.pt_eoff[gp];
                int fc_n = A.edge_fc[e0], cam_n = A.edge_cam[e0];
                Real z_n[2];
                obs_real(A, e0, z_n);
                for (int e = e0; e < e1; ++e) {
                    const int fc = fc_n, cam = cam_n;
                    const Real z[2] = {z_n[0], z_n[1]};
                    if (e + 1 < e1) {
                        fc_n = A.edge_fc[e + 1];
                        cam_n = A.edge_cam[e + 1];
                        obs_real(A, e + 1, z_n);
                    }
                    if (fc >= 0) {
                        Real cr[12];
                        cam_load(camr + 12 * cam, cr);
                        edge_jrec(A, e, cr, z, Xr, ltv, delta);
                    }
                }
                continue;
            }
        }
        for (int e = A.pt_eoff[gp]; e < e1; ++e) {
            if (A.edge_fc[e] < 0) continue;
            Real W[18];
            if (A.edge_w) {
                Rec<Real>::load18(A.edge_w + (long long)Rec<Real>::kEdge * e, W);
            } else {
                Real cr[12];
                cam_load(camr + 12 * A.edge_cam[e], cr);
                Real z[2];
                obs_real(A, e, z);
                EdgeLin<Real> L;
                edge_linearize_e<Real>(A, e, cr, Xr, z, delta, L);
#pragma unroll
                for (int r = 0; r < 6; ++r)
#pragma unroll
                    for (int k = 0; k < 3; ++k) W[r * 3 + k] = L.w * (L.jc[r] * L.jp[k] + L.jc[6 + r] * L.jp[3 + k]);
            }
            Real Ae[18];
#pragma unroll
            for (int r = 0; r < 6; ++r) {
                const Real w0 = W[r * 3 + 0], w1 = W[r * 3 + 1], w2 = W[r * 3 + 2];
                Ae[r * 3 + 0] = w0 * l00;
                Ae[r * 3 + 1] = w0 * l10 + w1 * l11;
                Ae[r * 3 + 2] = w0 * l20 + w1 * l21 + w2 * l22;
            }
            Rec<Real>::store18(A.edge_a + (long long)Rec<Real>::kEdge * e, Ae);
        }
    }
    return bad;
}

// Trial points dx_p = L^T (t_p - sum A_e^T dx_c); returns this thread's dx^T(lambda dx + g) part.
template <class Real, class DC>
__device__ double update_points(const WinArgs<Real>& A, const CC& c, const WinDesc& D, double lambda,
                                const DC* dcl, int cur) {
    const double* Xc = A.x[cur];
    double* Xt = A.x[cur ^ 1];
    Real* XRt = A.xr[cur ^ 1];
    const Real fx = (Real)A.intr.fx, fy = (Real)A.intr.fy;
    double sc = 0.0;
    for (int p = c.gt; p < D.npt; p += c.CT) {
        const int gp = D.pt0 + p;
        if (A.pt_free[gp] < 0) continue;
        Real lt[12];
        Rec<Real>::load12(A.pt_lt + 12LL * gp, lt);
        Real u0 = lt[6], u1 = lt[7], u2 = lt[8];
        const int e1 = A.pt_eoff[gp + 1];
        for (int e = A.pt_eoff[gp]; e < e1; ++e) {
            const int a = A.edge_fc[e];
            if (a >= 0) sub_at_d(A, e, dcl + 6 * a, fx, fy, u0, u1, u2);
        }
        // dx = L^T u
        const Real d0 = lt[0] * u0 + lt[1] * u1 + lt[3] * u2;
        const Real d1 = lt[2] * u1 + lt[4] * u2;
        const Real d2 = lt[5] * u2;
        store_trial_point(Xc, Xt, XRt, gp, d0, d1, d2);
        Real vg[12];
        Rec<Real>::load12(A.pt_vg + 12LL * gp, vg);
        sc += (double)d0 * (lambda * (double)d0 + (double)vg[6]) + (double)d1 * (lambda * (double)d1 + (double)vg[7]) +
              (double)d2 * (lambda * (double)d2 + (double)vg[8]);
    }
    return sc;
}

// Mixed form: the trial points of update_points fused with the trial cost change.  For every edge
// of the window's points the residual change is formed from the state change, in Real, without
// cancellation against the pixel coordinates:
//   Xc' - Xc = (E - I)(Xc + R dX) + R dX + E_t     (E, E_t: the camera's step exp(dx_c), camdel)
//   dpi = pi(Xc') - pi(Xc) = f (dx z - x dz) / (z z'),   e' = e - dpi,
//   d rho = ds = -dpi . (e + e')  (both quadratic),  2 delta ds / (sqrt s' + sqrt s)  (both Huber),
// so each d rho carries Real's relative precision of the change itself, not of the pixel values.
// e of the current state is read from edge_e[cur], e' written to edge_e[cur ^ 1].  Pinhole model.
// Returns (this thread's dx^T(lambda dx + g) part, its Kahan-compensated d chi part).
template <class Real>
__device__ double2 update_points_dcost(const WinArgs<Real>& A, const CC& c, const WinDesc& D, double lambda,
                                       const Real* dcl, int cur, const Real* camr, const Real* camdel) {
    const double* Xc = A.x[cur];
    double* Xt = A.x[cur ^ 1];
    const Real* XRc = A.xr[cur];
    Real* XRt = A.xr[cur ^ 1];
    const Real* ecur = A.edge_e[cur];
    Real* etr = A.edge_e[cur ^ 1];
    const Real fx = (Real)A.intr.fx, fy = (Real)A.intr.fy;
    const bool robust = A.lm.robust != 0;
    const Real hd = (Real)A.lm.huber_delta, hd2 = hd * hd;
    const Real lam = (Real)lambda;
    double sc = 0.0;
    Real ks = Real(0), kc = Real(0);
    for (int p = c.gt; p < D.npt; p += c.CT) {
        const int gp = D.pt0 + p;
        const bool fp = A.pt_free[gp] >= 0;
        Real d0 = Real(0), d1 = Real(0), d2 = Real(0);
        const int e0i = A.pt_eoff[gp], e1i = A.pt_eoff[gp + 1];
        if (fp) {
            Real lt[12];
            Rec<Real>::load12(A.pt_lt + 12LL * gp, lt);
            Real u0 = lt[6], u1 = lt[7], u2 = lt[8];
            bool done = false;
            if constexpr (sizeof(Real) == 4) {
              if (A.jfact) {
                // Jacobian-factored records: the next edge's record and free camera are loaded before
                // the current edge's products (a fixed camera's record is loaded and not used)
                Real rec[12], nrec[12];
                int a_n = A.edge_fc[e0i];
                JRec::load(A.edge_a + (long long)JRec::kEdge * e0i, nrec);
                for (int e = e0i; e < e1i; ++e) {
                    const int a = a_n;
#pragma unroll
                    for (int k = 0; k < 12; ++k) rec[k] = nrec[k];
                    if (e + 1 < e1i) {
                        a_n = A.edge_fc[e + 1];
                        JRec::load(A.edge_a + (long long)JRec::kEdge * (e + 1), nrec);
                    }
                    if (a >= 0) sub_at_d_rec(rec, dcl + 6 * a, fx, fy, u0, u1, u2);
                }
                done = true;
              }
            }
            if (!done)
                for (int e = e0i; e < e1i; ++e) {
                    const int a = A.edge_fc[e];
                    if (a >= 0) sub_at_d(A, e, dcl + 6 * a, fx, fy, u0, u1, u2);
                }
            d0 = lt[0] * u0 + lt[1] * u1 + lt[3] * u2;
            d1 = lt[2] * u1 + lt[4] * u2;
            d2 = lt[5] * u2;
            store_trial_point(Xc, Xt, XRt, gp, d0, d1, d2);
            Real vg[12];
            Rec<Real>::load12(A.pt_vg + 12LL * gp, vg);
            // the point's model-decrease term in Real (its relative error is Real's; the terms are
            // summed in FP64)
            sc += (double)(d0 * (lam * d0 + vg[6]) + d1 * (lam * d1 + vg[7]) + d2 * (lam * d2 + vg[8]));
        }
        Real X[3];
        point_real(Xc, XRc, gp, X);
        // the next edge's camera and current residual are loaded before this edge's products
        int cam_n = e0i < e1i ? A.edge_cam[e0i] : 0;
        Real r0_n = e0i < e1i ? ecur[2LL * e0i] : Real(0), r1_n = e0i < e1i ? ecur[2LL * e0i + 1] : Real(0);
        for (int e = e0i; e < e1i; ++e) {
            const int cam = cam_n;
            const Real r0 = r0_n, r1 = r1_n;
            if (e + 1 < e1i) {
                cam_n = A.edge_cam[e + 1];
                r0_n = ecur[2LL * e + 2];
                r1_n = ecur[2LL * e + 3];
            }
            Real cr[12], cd[12];
            cam_load(camr + 12 * cam, cr);
            cam_load(camdel + 12 * cam, cd);
            Real xc[3];
            transform(cr, cr + 9, X, xc);
            const Real rd[3] = {cr[0] * d0 + cr[1] * d1 + cr[2] * d2, cr[3] * d0 + cr[4] * d1 + cr[5] * d2,
                                cr[6] * d0 + cr[7] * d1 + cr[8] * d2};
            const Real q[3] = {xc[0] + rd[0], xc[1] + rd[1], xc[2] + rd[2]};
            Real dx[3];
#pragma unroll
            for (int i = 0; i < 3; ++i) dx[i] = cd[3 * i] * q[0] + cd[3 * i + 1] * q[1] + cd[3 * i + 2] * q[2] + rd[i] + cd[9 + i];
            const Real z = xc[2], zt = z + dx[2];
            const Real inv = Real(1) / (z * zt);
            const Real dpu = fx * (dx[0] * z - xc[0] * dx[2]) * inv;
            const Real dpv = fy * (dx[1] * z - xc[1] * dx[2]) * inv;
            const Real n0 = r0 - dpu, n1 = r1 - dpv;
            etr[2LL * e] = n0;
            etr[2LL * e + 1] = n1;
            const Real ds = -(dpu * (r0 + n0) + dpv * (r1 + n1));
            Real dr = ds;
            if (robust) {
                const Real s = r0 * r0 + r1 * r1, sn = n0 * n0 + n1 * n1;
                if (s > hd2 && sn > hd2) {
                    dr = Real(2) * hd * ds / (sqrt(sn) + sqrt(s));
                } else if (s > hd2 || sn > hd2) {
                    const Real rho_o = s > hd2 ? Real(2) * hd * sqrt(s) - hd2 : s;
                    const Real rho_n = sn > hd2 ? Real(2) * hd * sqrt(sn) - hd2 : sn;
                    dr = rho_n - rho_o;
                }
            }
            const Real y = dr - kc;
            const Real t = ks + y;
            kc = (t - ks) - y;
            ks = t;
        }
    }
    return make_double2(sc, (double)ks - (double)kc);
}

}  // namespace
}  // namespace navba
