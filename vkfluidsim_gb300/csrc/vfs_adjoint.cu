// Reverse-mode (adjoint) kernels of the WCSPH substep and the checkpointed rollout around them.
//
// The forward substep (src/models/wcsph_with_boundary_model.cpp:93-116; shaders
// wcsph_with_boundary_model.slang:102-360) is differentiated as a smooth function of the sorted
// positions x', velocities v', viscosity nu and stiffness k: neighbour sets, the sort and branch
// choices are piecewise constant and carry no gradient. Notation, per ordered pair (i, j) of the
// density pass's neighbour list, x = x_i - x_j, r = |x|, n = x / r, gw = the shader's kernel
// gradient (with its extra 1/h), W = the cubic spline, c = adjoint of a_i:
//   pressure   a_i -= m (pd_i + pd_j) gw(r) n          -> d(-c.T)/dx, d/dpd_i, d/dpd_j
//   viscosity  a_i += 10 nu mr_j (v_ij.x) gw(r) n / (r^2 + 0.01 h^2)
//   boundary   a_i -= (pd_i + pb_i) rho0 G_i, rho_i += rho0 Psi_i (volume-map terms)
//   wall       a_i -= k_w diff(x_i)
//   EOS        pd = p / rho^2, pb = p / rho0^2, mr = m / max(rho, 1e-6), p = k ((rho/rho0)^g - 1)
//   density    rho_i = sum_j m W(r_ij) + rho0 Psi_i
// Pair contributions to the other particle j are scattered with atomics (the list of i holds j
// with the reference's multiplicity, which need not be symmetric under hash collisions).
#include <cuda_runtime.h>

#include <cmath>
#include <string>
#include <vector>

#include "vfs_cuda.h"
#include "vfs_internal.h"
#include "vfs_model.h"

namespace vfs {
namespace {

constexpr uint32_t kErrAdjointOverflow = 2u;  // a neighbour list longer than its capacity
constexpr int kAdjLanes = 4;                     // lanes sharing one particle's neighbour list

__device__ __forceinline__ float3 f3(const float4& a) { return make_float3(a.x, a.y, a.z); }
__device__ __forceinline__ float dot3(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ float3 operator+(float3 a, float3 b) { return make_float3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ float3 operator-(float3 a, float3 b) { return make_float3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ float3 operator*(float s, float3 a) { return make_float3(s * a.x, s * a.y, s * a.z); }

// One 16-byte vector atomic (sm_90 and later) instead of three scalar ones.
__device__ __forceinline__ void atomic_add3(float4* p, float3 v) {
    atomicAdd(p, make_float4(v.x, v.y, v.z, 0.0f));
}

// Shader kernel gradient gw(r) and its derivative d gw / dr (kernels_3d.slang:78-91).
__device__ __forceinline__ void gw_and_deriv(const SceneParams& p, float r, float& gw, float& dgw) {
    const float q = r * p.inv_h;
    gw = 0.0f;
    dgw = 0.0f;
    if (r > 1e-9f && q <= 1.0f) {
        const float G = p.grad_over_h;
        if (q > 0.5f) {
            const float t = 1.0f - q;
            gw = -G * t * t;
            dgw = 2.0f * G * t * p.inv_h;
        } else {
            gw = G * q * (3.0f * q - 2.0f);
            dgw = G * (6.0f * q - 2.0f) * p.inv_h;
        }
    }
}

// dW/dr of the cubic spline (kernels_3d.slang:62-76): h * gw(r) inside the support.
__device__ __forceinline__ float dW_dr(const SceneParams& p, float r) {
    float gw, dgw;
    gw_and_deriv(p, r, gw, dgw);
    return p.h * gw;
}

__device__ __forceinline__ float cubic_W(const SceneParams& p, float r) {
    const float q = r * p.inv_h;
    if (q > 1.0f) return 0.0f;
    if (q > 0.5f) {
        const float t = 1.0f - q;
        return p.cubic * 2.0f * t * t * t;
    }
    return p.cubic * (6.0f * q * q * q - 6.0f * q * q + 1.0f);
}

// ---- trilinear grid sampling with its gradient (SampleGrid, slang:51-66, cells clamped) ----

struct GridSample {
    float v;
    float3 g;  // d value / d local coordinates
};

__device__ __forceinline__ GridSample sample_grad(const float* __restrict__ grid, const DevObject& o,
                                                  float3 l) {
    const float u[3] = {(l.x - o.box_pos[0]) / o.box_size[0], (l.y - o.box_pos[1]) / o.box_size[1],
                        (l.z - o.box_pos[2]) / o.box_size[2]};
    uint32_t cell[3];
    float chi[3], dchi[3];
    for (int a = 0; a < 3; a++) {
        const uint32_t n = o.res[a];
        const float x = ((float)n - 1.0f) * u[a];
        float f = floorf(x);
        if (!(f >= 0.0f)) f = 0.0f;
        if (f > (float)(n - 2u)) f = (float)(n - 2u);
        cell[a] = (uint32_t)f;
        chi[a] = 2.0f * (x - f) - 1.0f;
        dchi[a] = 2.0f * ((float)n - 1.0f) / o.box_size[a];  // d chi / d local
    }
    const size_t sy = o.res[0], sz = (size_t)o.res[0] * o.res[1];
    const size_t b = cell[0] + sy * cell[1] + sz * cell[2];
    float v = 0.0f, gx = 0.0f, gy = 0.0f, gz = 0.0f;
#pragma unroll
    for (int i = 0; i < 8; i++) {
        const int ox = i >> 2, oy = i & 1, oz = (i >> 1) & 1;
        const float sx = ox ? 1.0f : -1.0f, sy_ = oy ? 1.0f : -1.0f, sz_ = oz ? 1.0f : -1.0f;
        const float fx = 1.0f + sx * chi[0], fy = 1.0f + sy_ * chi[1], fz = 1.0f + sz_ * chi[2];
        const float gval = __ldg(grid + b + ox + oy * sy + oz * sz);
        v += gval * fx * fy * fz;
        gx += gval * sx * fy * fz;
        gy += gval * fx * sy_ * fz;
        gz += gval * fx * fy * sz_;
    }
    GridSample s;
    s.v = v * 0.125f;
    s.g = make_float3(gx * 0.125f * dchi[0], gy * 0.125f * dchi[1], gz * 0.125f * dchi[2]);
    return s;
}

__device__ __forceinline__ float3 mat3_row_apply(const float* M, float3 v) {  // rows of a 3x4
    return make_float3(M[0] * v.x + M[1] * v.y + M[2] * v.z, M[4] * v.x + M[5] * v.y + M[6] * v.z,
                       M[8] * v.x + M[9] * v.y + M[10] * v.z);
}
__device__ __forceinline__ float3 mat3_T_apply(const float* M, float3 v) {  // transpose of a 3x4
    return make_float3(M[0] * v.x + M[4] * v.y + M[8] * v.z, M[1] * v.x + M[5] * v.y + M[9] * v.z,
                       M[2] * v.x + M[6] * v.y + M[10] * v.z);
}

// Adjoint of CalculateBoundaryVolume (slang:102-151) for one particle: returns d L / d x given
// psi_bar = d L / d Psi_i and G_bar = d L / d G_i.
__device__ float3 boundary_adjoint(const SceneParams& p, float3 x, float psi_bar, float3 G_bar) {
    float3 xbar = make_float3(0.f, 0.f, 0.f);
    for (uint32_t oi = 0; oi < p.n_objects; oi++) {
        const DevObject& o = p.objects[oi];
        const float3 l = make_float3(o.T[0] * x.x + o.T[1] * x.y + o.T[2] * x.z + o.T[3],
                                     o.T[4] * x.x + o.T[5] * x.y + o.T[6] * x.z + o.T[7],
                                     o.T[8] * x.x + o.T[9] * x.y + o.T[10] * x.z + o.T[11]);
        if (l.x < o.box_pos[0] || l.y < o.box_pos[1] || l.z < o.box_pos[2] ||
            l.x > o.box_pos[0] + o.box_size[0] || l.y > o.box_pos[1] + o.box_size[1] ||
            l.z > o.box_pos[2] + o.box_size[2])
            continue;
        const GridSample S = sample_grad(o.sdf, o, l);
        if (!(S.v >= 0.0f && S.v < p.h)) continue;
        const GridSample V = sample_grad(o.vm, o, l);
        if (!(V.v > 0.0f)) continue;
        const float e = p.grad_eps;
        const float3 ex = make_float3(e, 0.f, 0.f), ey = make_float3(0.f, e, 0.f),
                     ez = make_float3(0.f, 0.f, e);
        const GridSample sxp = sample_grad(o.sdf, o, l + ex), sxm = sample_grad(o.sdf, o, l - ex);
        const GridSample syp = sample_grad(o.sdf, o, l + ey), sym = sample_grad(o.sdf, o, l - ey);
        const GridSample szp = sample_grad(o.sdf, o, l + ez), szm = sample_grad(o.sdf, o, l - ez);
        const float inv2e = 1.0f / (2.0f * e);
        const float3 g = make_float3((sxp.v - sxm.v) * inv2e, (syp.v - sym.v) * inv2e,
                                     (szp.v - szm.v) * inv2e);
        const float modn = sqrtf(dot3(g, g));
        if (!(modn > 1e-9f)) continue;
        const float3 ghat = (1.0f / modn) * g;
        const float3 nrm = mat3_row_apply(o.R, ghat);
        const bool d_active = S.v + p.bnd_eighth > p.bnd_half;
        const float d = d_active ? S.v + p.bnd_eighth : p.bnd_half;
        float gw, dgw;
        gw_and_deriv(p, d, gw, dgw);
        const float Wd = cubic_W(p, d);
        const float dWd = p.h * gw;
        const float3 grad_d = d_active ? S.g : make_float3(0.f, 0.f, 0.f);
        // d Psi / d l = W(d) grad V + V W'(d) grad d.
        float3 lbar = psi_bar * (Wd * V.g + (V.v * dWd) * grad_d);
        // G = V gw(d) n: (G_bar . n)(gw grad V + V gw' grad d) + V gw (dn/dl)^T G_bar.
        const float gn = dot3(G_bar, nrm);
        lbar = lbar + gn * (gw * V.g + (V.v * dgw) * grad_d);
        const float3 rg = mat3_T_apply(o.R, G_bar);         // R^T G_bar
        const float3 w = (1.0f / modn) * (rg - dot3(rg, ghat) * ghat);  // (I - gg^T)/|g| R^T G_bar
        // J_g^T w with J_g[a][b] = (dS/dl_b(l + e e_a) - dS/dl_b(l - e e_a)) / 2e.
        const float3 jt = (w.x * inv2e) * (sxp.g - sxm.g) + (w.y * inv2e) * (syp.g - sym.g) +
                          (w.z * inv2e) * (szp.g - szm.g);
        lbar = lbar + (V.v * gw) * jt;
        xbar = xbar + mat3_T_apply(o.T, lbar);  // d l / d x = T (linear part)
    }
    return xbar;
}

// ---- the reverse substep, one thread per sorted particle ----

struct AdjBuffers {
    const float4* pos;   // x' (sorted positions of the substep)
    const float4* vel;   // v'
    const float4* aux;   // (pd, mr, rho, pb)
    const float4* bnd;   // (G, Psi)
    const uint32_t* nbr;
    const uint32_t* nbr_count;
    float4* xbar;        // accumulates d L / d x' (sorted order)
    float4* vbar;        // accumulates d L / d v'
    float4* abar;        // d L / d a
    float2* pmbar;       // (d L / d pd, d L / d mr)
    float* pbbar;
    float* rhobar;
    float4* gbar;        // d L / d G
    double* dparams;     // [d nu, d k]
    uint32_t* err;
};

// Symplectic Euler, reversed: x_out = x' + v_out dt, v_out = v' + a dt.
__global__ void k_adj_integrate(SceneParams p, uint32_t n, const float4* __restrict__ xbar_out,
                                const float4* __restrict__ vbar_out, AdjBuffers B) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 xo = xbar_out[i], vo = vbar_out[i];
    const float vx = vo.x + p.dt * xo.x, vy = vo.y + p.dt * xo.y, vz = vo.z + p.dt * xo.z;
    B.xbar[i] = make_float4(xo.x, xo.y, xo.z, 0.f);
    B.vbar[i] = make_float4(vx, vy, vz, 0.f);
    B.abar[i] = make_float4(p.dt * vx, p.dt * vy, p.dt * vz, 0.f);
    B.pmbar[i] = make_float2(0.f, 0.f);
}

// Sums v over the block and adds it to *dst with one atomic (one address is shared by the whole
// grid, so per-warp atomics would serialise). Every thread of the block must call it.
__device__ __forceinline__ void block_add_double(double v, double* dst) {
    __shared__ double s_part[32];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) s_part[warp] = v;
    __syncthreads();
    if (warp == 0) {
        const int nw = (blockDim.x + 31) >> 5;
        double t = lane < nw ? s_part[lane] : 0.0;
        for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
        if (lane == 0 && t != 0.0) atomicAdd(dst, t);
    }
}

// Sums v over the kLanes lanes of a particle group (consecutive lanes of one warp). Every lane of
// the warp must call it.
template <int kLanes>
__device__ __forceinline__ float group_sum(float v) {
#pragma unroll
    for (int o = kLanes / 2; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

template <int kLanes>
__device__ __forceinline__ float3 group_sum3(float3 v) {
    return make_float3(group_sum<kLanes>(v.x), group_sum<kLanes>(v.y), group_sum<kLanes>(v.z));
}

// Adjoint of the force pass: pressure, viscosity, boundary pressure and wall terms.
//
// Pair (j, i) of j's force, with x = x_j - x_i, v = v_j - v_i, n = x / r, c_j = d L / d a_j:
//   pressure  L-term -m (pd_j + pd_i) gw(r) (c_j . n)
//   viscosity L-term  s_i (v . x)(c_j . x) u(r),  s_i = 10 nu mr_i,  u = gw / (r (r^2 + eps)).
// Both are linear in c_j, and pair (i, j) of i's force is the same expression with c_i, s_j and
// (x, v) negated. Particle j's list is split over kLanes lanes. When i and j both have distinct
// neighbour keys and adjacent cells, each lists the other exactly once, so j also gathers the part
// of pair (i, j) that falls on j, which is the own-pair expression evaluated at c_j - c_i (pressure)
// and s_i c_j - s_j c_i (viscosity). Otherwise i's part is left to i, which scatters its own
// pair's reverse to j with atomics (c_i counted as zero here).
template <int kLanes>
__global__ void __launch_bounds__(128) k_adj_force(SceneParams p, uint32_t n, AdjBuffers B) {
    const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t j = (uint32_t)(t / kLanes), lane = (uint32_t)(t % kLanes);
    float3 xb = make_float3(0.f, 0.f, 0.f), vb = make_float3(0.f, 0.f, 0.f);
    float pdb = 0.f, mrb = 0.f, dnu_f = 0.f;
    float3 xj = xb, cj = xb;
    float pdj = 0.f, pbj = 0.f;
    if (j < n) {
        xj = f3(B.pos[j]);
        const float3 vj = f3(B.vel[j]);
        const float4 aj = B.aux[j];
        cj = f3(B.abar[j]);
        pdj = aj.x;
        pbj = aj.w;
        const float s_j = p.visc_scale * aj.y;
        const uint32_t cnt = B.nbr_count[j];
        const bool dj = (cnt & kNbrDistinct) != 0u;
        if (lane == 0 && (cnt & kNbrCountMask) > p.nbr_cap) atomicOr(B.err, kErrAdjointOverflow);
        const uint32_t listed = min(cnt & kNbrCountMask, p.nbr_cap);
        for (uint32_t k = lane; k < listed; k += kLanes) {
            const uint32_t i = B.nbr[(size_t)k * n + j];
            const float3 x = xj - f3(B.pos[i]);
            const float r2 = dot3(x, x);
            if (!(r2 > 1e-18f)) continue;
            const float inv_r = rsqrtf(r2);
            const float r = r2 * inv_r;
            const float3 v = vj - f3(B.vel[i]);
            const float2 ai = *reinterpret_cast<const float2*>(B.aux + i);  // (pd_i, mr_i)
            const uint32_t ci_word = B.nbr_count[i];
            const bool gather = dj && (ci_word & kNbrDistinct) != 0u && nbr_cells_adjacent(cnt, ci_word);
            const float3 ci = gather ? f3(B.abar[i]) : make_float3(0.f, 0.f, 0.f);
            float gw, dgw;
            gw_and_deriv(p, r, gw, dgw);
            const float inv_den = 1.0f / (r2 + p.visc_eps);
            const float u = gw * inv_r * inv_den;
            const float du = (dgw * r - gw * (3.0f * r2 + p.visc_eps) * inv_den) * inv_r * inv_r * inv_den;
            const float s_i = p.visc_scale * ai.y;
            const float3 nn = inv_r * x;
            const float3 dc = cj - ci;
            const float3 cv = s_i * cj - s_j * ci;
            const float dcn = dot3(dc, nn), cvx = dot3(cv, x), vx = dot3(v, x), cjx = dot3(cj, x);
            const float3 dx = (-p.mass * (pdj + ai.x)) * ((dgw * dcn) * nn + (gw * inv_r) * (dc - dcn * nn)) +
                              (cvx * u) * v + (vx * u) * cv + (vx * cvx * du) * nn;
            const float3 dv = (cvx * u) * x;
            const float dp = -p.mass * gw * dcn;
            xb = xb + dx;
            vb = vb + dv;
            pdb += dp;
            dnu_f += ai.y * vx * cjx * u;
            if (gather) {
                mrb -= p.visc_scale * vx * dot3(ci, x) * u;
            } else {
                atomic_add3(&B.xbar[i], -1.0f * dx);
                atomic_add3(&B.vbar[i], -1.0f * dv);
                atomicAdd(&B.pmbar[i], make_float2(dp, p.visc_scale * vx * cjx * u));
            }
        }
    }
    xb = group_sum3<kLanes>(xb);
    vb = group_sum3<kLanes>(vb);
    pdb = group_sum<kLanes>(pdb);
    mrb = group_sum<kLanes>(mrb);
    if (j < n && lane == 0) {
        // Boundary pressure: L-term = -(pd_j + pb_j) rho0 (c . G_j).
        const float3 G = f3(B.bnd[j]);
        const float cg = dot3(cj, G);
        pdb += -p.rho0 * cg;
        B.pbbar[j] = -p.rho0 * cg;
        const float sg = -(pdj + pbj) * p.rho0;
        B.gbar[j] = make_float4(sg * cj.x, sg * cj.y, sg * cj.z, 0.f);
        // Wall penalty: a -= k_w diff(x), d diff / dx = 1 outside [lo, hi].
        const float xs[3] = {xj.x, xj.y, xj.z};
        const float cs[3] = {cj.x, cj.y, cj.z};
        float wb[3];
        for (int a = 0; a < 3; a++)
            wb[a] = (xs[a] < p.lo[a] || xs[a] > p.hi[a]) ? -p.wall_k * cs[a] : 0.0f;
        xb = xb + make_float3(wb[0], wb[1], wb[2]);
        atomic_add3(&B.xbar[j], xb);
        atomic_add3(&B.vbar[j], vb);
        atomicAdd(&B.pmbar[j], make_float2(pdb, mrb));
    }
    block_add_double(10.0 * (double)dnu_f, &B.dparams[0]);
}

// Adjoint of the EOS epilogue: rho_bar from pd_bar, pb_bar, mr_bar; d L / d k.
__global__ void k_adj_eos(SceneParams p, uint32_t n, AdjBuffers B) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    float dk = 0.0f;
    if (i < n) {
        const float4 ai = B.aux[i];
        const float rho = ai.z;
        const float inv_rho0 = 1.0f / p.rho0;
        const float ratio = fmaxf(rho, p.rho0) * inv_rho0;
        const float pw = powf(ratio, p.expoent);  // ratio^gamma
        const float f = pw - 1.0f;                // p = k f
        const float pr = p.stiffness * f;
        const float dp = rho > p.rho0 ? p.stiffness * p.expoent * pw / fmaxf(rho, p.rho0) : 0.0f;
        const float2 pm = B.pmbar[i];
        const float pdb = pm.x, pbb = B.pbbar[i], mrb = pm.y;
        const float inv_rho = rho > 0.0f ? 1.0f / rho : 0.0f;
        float rb = pdb * (dp - 2.0f * pr * inv_rho) * inv_rho * inv_rho;
        rb += pbb * dp * inv_rho0 * inv_rho0;
        if (rho > 1e-6f) rb -= mrb * p.mass * inv_rho * inv_rho;
        B.rhobar[i] = rb;
        dk = (pdb * inv_rho * inv_rho + pbb * inv_rho0 * inv_rho0) * f;
    }
    block_add_double((double)dk, &B.dparams[1]);
}

// Adjoint of the density sum and of the volume-map terms, the list split over kLanes lanes as in
// k_adj_force; the reverse half of each pair is gathered or scattered under the same rule.
template <int kLanes>
__global__ void __launch_bounds__(128) k_adj_density(SceneParams p, uint32_t n, AdjBuffers B) {
    const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t j = (uint32_t)(t / kLanes), lane = (uint32_t)(t % kLanes);
    float3 xb = make_float3(0.f, 0.f, 0.f), xj = xb;
    float rbj = 0.0f;
    if (j < n) {
        xj = f3(B.pos[j]);
        rbj = B.rhobar[j];
        const uint32_t cnt = B.nbr_count[j];
        const bool dj = (cnt & kNbrDistinct) != 0u;
        const uint32_t listed = min(cnt & kNbrCountMask, p.nbr_cap);
        for (uint32_t k = lane; k < listed; k += kLanes) {
            const uint32_t i = B.nbr[(size_t)k * n + j];
            const float3 x = xj - f3(B.pos[i]);
            const float r2 = dot3(x, x);
            if (!(r2 > 1e-18f)) continue;
            const float inv_r = rsqrtf(r2);
            const float w = p.mass * dW_dr(p, r2 * inv_r) * inv_r;
            const uint32_t ci_word = B.nbr_count[i];
            const bool gather = dj && (ci_word & kNbrDistinct) != 0u && nbr_cells_adjacent(cnt, ci_word);
            // Own pair: d rho_j / d x_j = m W'(r) n, d rho_j / d x_i = -m W'(r) n.
            if (gather)
                xb = xb + ((rbj + B.rhobar[i]) * w) * x;  // with i's pair (i, j): d rho_i / d x_j
            else {
                xb = xb + (rbj * w) * x;
                if (rbj != 0.0f) atomic_add3(&B.xbar[i], (-rbj * w) * x);
            }
        }
    }
    xb = group_sum3<kLanes>(xb);
    if (j < n && lane == 0) {
        const float4 gb = B.gbar[j];
        const float psib = rbj * p.rho0;
        if (p.n_objects && (psib != 0.0f || gb.x != 0.0f || gb.y != 0.0f || gb.z != 0.0f))
            xb = xb + boundary_adjoint(p, xj, psib, f3(gb));
        atomic_add3(&B.xbar[j], xb);
    }
}

// Back through the reorder x' = x[perm]: scatter into the previous order.
__global__ void k_adj_unsort(uint32_t n, const uint32_t* __restrict__ perm,
                             const float4* __restrict__ xs, const float4* __restrict__ vs,
                             float4* __restrict__ xprev, float4* __restrict__ vprev) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t src = perm[i];
    if (src >= n) return;
    xprev[src] = xs[i];
    vprev[src] = vs[i];
}

// Places a by-id host gradient onto the particles of a state whose ids are in pos.w.
__global__ void k_adj_by_id(uint32_t n, const float4* __restrict__ pos, const float* __restrict__ g3,
                            float4* __restrict__ out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t id = __float_as_uint(pos[i].w);
    out[i] = id < n && g3 ? make_float4(g3[3 * id], g3[3 * id + 1], g3[3 * id + 2], 0.f)
                          : make_float4(0.f, 0.f, 0.f, 0.f);
}

// Gathers a per-particle float4 field into by-id float3 order.
__global__ void k_to_id(uint32_t n, const float4* __restrict__ pos, const float4* __restrict__ f,
                        float* __restrict__ out3) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t id = __float_as_uint(pos[i].w);
    if (id >= n) return;
    out3[3 * id] = f[i].x;
    out3[3 * id + 1] = f[i].y;
    out3[3 * id + 2] = f[i].z;
}

}  // namespace

#define VFS_ADJ_TRY(expr)                                                                 \
    do {                                                                                  \
        cudaError_t e_ = (expr);                                                          \
        if (e_ != cudaSuccess)                                                            \
            return ::vfs::fail(VFS_ERR_CUDA, std::string(#expr) + ": " + cudaGetErrorString(e_)); \
    } while (0)

// A checkpointed differentiable rollout of a single-scene model.
struct Rollout {
    Model* m = nullptr;
    int steps = 0, every = 0;
    std::vector<float4*> ck_pos, ck_vel;  // state before steps 0, every, 2 every, ...
    float4 *fin_pos = nullptr, *fin_vel = nullptr;  // state after the last step
    // One segment of per-substep records.
    std::vector<float4*> s_pos, s_vel, s_aux, s_bnd;
    std::vector<uint32_t*> s_perm, s_nbr, s_cnt;
    float4 *xbar = nullptr, *vbar = nullptr, *xs = nullptr, *vs = nullptr, *abar = nullptr, *gbar = nullptr;
    float2* pmbar = nullptr;
    float *pbbar = nullptr, *rhobar = nullptr;
    float* host_io = nullptr;  // 3N floats on the device for host transfers
    double* dparams = nullptr;
    bool forward_done = false;
    uint32_t cap = 0;  // neighbour slots per particle of the segment records (the model's at creation)
    bool last_recorded = false;  // the segment records hold the last segment (set by forward)
    cudaGraphExec_t seg_graph = nullptr;  // recompute + reverse of one full segment

    ~Rollout() {
        if (seg_graph) cudaGraphExecDestroy(seg_graph);
        for (auto* p : ck_pos) cudaFree(p);
        for (auto* p : ck_vel) cudaFree(p);
        for (auto* p : s_pos) cudaFree(p);
        for (auto* p : s_vel) cudaFree(p);
        for (auto* p : s_aux) cudaFree(p);
        for (auto* p : s_bnd) cudaFree(p);
        for (auto* p : s_perm) cudaFree(p);
        for (auto* p : s_nbr) cudaFree(p);
        for (auto* p : s_cnt) cudaFree(p);
        cudaFree(fin_pos);
        cudaFree(fin_vel);
        cudaFree(xbar);
        cudaFree(vbar);
        cudaFree(xs);
        cudaFree(vs);
        cudaFree(abar);
        cudaFree(gbar);
        cudaFree(pmbar);
        cudaFree(pbbar);
        cudaFree(rhobar);
        cudaFree(host_io);
        cudaFree(dparams);
    }

    int init(Model* model, int n_steps, int ck_every) {
        m = model;
        cap = m->nbr_cap;
        steps = n_steps;
        every = ck_every < 1 ? 1 : ck_every;
        const size_t N = m->n ? m->n : 1;
        const int n_ck = (steps + every - 1) / every;
        ck_pos.resize(n_ck, nullptr);
        ck_vel.resize(n_ck, nullptr);
        for (int c = 0; c < n_ck; c++) {
            VFS_ADJ_TRY(cudaMalloc(&ck_pos[c], N * sizeof(float4)));
            VFS_ADJ_TRY(cudaMalloc(&ck_vel[c], N * sizeof(float4)));
        }
        const int seg = every < steps ? every : steps;
        s_pos.resize(seg, nullptr);
        s_vel.resize(seg, nullptr);
        s_aux.resize(seg, nullptr);
        s_bnd.resize(seg, nullptr);
        s_perm.resize(seg, nullptr);
        s_nbr.resize(seg, nullptr);
        s_cnt.resize(seg, nullptr);
        for (int t = 0; t < seg; t++) {
            VFS_ADJ_TRY(cudaMalloc(&s_pos[t], N * sizeof(float4)));
            VFS_ADJ_TRY(cudaMalloc(&s_vel[t], N * sizeof(float4)));
            VFS_ADJ_TRY(cudaMalloc(&s_aux[t], N * sizeof(float4)));
            VFS_ADJ_TRY(cudaMalloc(&s_bnd[t], N * sizeof(float4)));
            VFS_ADJ_TRY(cudaMalloc(&s_perm[t], N * 4));
            VFS_ADJ_TRY(cudaMalloc(&s_nbr[t], N * (size_t)cap * 4));
            VFS_ADJ_TRY(cudaMalloc(&s_cnt[t], N * 4));
        }
        for (float4** b : {&fin_pos, &fin_vel, &xbar, &vbar, &xs, &vs, &abar, &gbar})
            VFS_ADJ_TRY(cudaMalloc(b, N * sizeof(float4)));
        for (float** b : {&pbbar, &rhobar}) VFS_ADJ_TRY(cudaMalloc(b, N * 4));
        VFS_ADJ_TRY(cudaMalloc(&pmbar, N * sizeof(float2)));
        VFS_ADJ_TRY(cudaMalloc(&host_io, N * 12));
        VFS_ADJ_TRY(cudaMalloc(&dparams, 2 * sizeof(double)));
        return VFS_OK;
    }

    int save(float4* dp, float4* dv) {
        const size_t bytes = (size_t)m->n * sizeof(float4);
        VFS_ADJ_TRY(cudaMemcpyAsync(dp, m->pos[m->cur], bytes, cudaMemcpyDeviceToDevice, m->stream));
        VFS_ADJ_TRY(cudaMemcpyAsync(dv, m->vel[m->cur], bytes, cudaMemcpyDeviceToDevice, m->stream));
        return VFS_OK;
    }
    int restore(const float4* dp, const float4* dv) {
        const size_t bytes = (size_t)m->n * sizeof(float4);
        VFS_ADJ_TRY(cudaMemcpyAsync(m->pos[m->cur], dp, bytes, cudaMemcpyDeviceToDevice, m->stream));
        VFS_ADJ_TRY(cudaMemcpyAsync(m->vel[m->cur], dv, bytes, cudaMemcpyDeviceToDevice, m->stream));
        return VFS_OK;
    }

    // First substep of the last segment, and its length.
    int last_t0() const { return ((steps - 1) / every) * every; }
    int last_len() const { return steps - last_t0(); }

    // Runs the rollout from the model's state, saving a checkpoint every `every` substeps. The last
    // segment is recorded as it runs, so the adjoint starts without recomputing it.
    int forward() {
        forward_done = false;
        const int t_last = last_t0();
        for (int t = 0; t < t_last; t++) {
            if (t % every == 0) {
                const int rc = save(ck_pos[t / every], ck_vel[t / every]);
                if (rc) return rc;
            }
            const int rc = m->run_substeps(1);
            if (rc) return rc;
        }
        int rc = save(ck_pos[t_last / every], ck_vel[t_last / every]);
        if (rc == VFS_OK) rc = record_segment(last_len());
        if (rc == VFS_OK) rc = save(fin_pos, fin_vel);
        if (rc) return rc;
        rc = m->check_device();
        if (rc) return rc;
        forward_done = true;
        last_recorded = true;
        return VFS_OK;
    }

    // Recomputes `len` substeps from the state in the model, keeping each substep's sorted inputs,
    // permutation, density products and neighbour lists: the model's buffers for those are pointed
    // at the segment's per-substep records, so the passes write them in place.
    int record_segment(int len) {
        if (m->nbr_cap != cap)
            return fail(VFS_ERR_INVALID_ARGUMENT, "the model's neighbour capacity changed after the rollout was created");
        float4* own_aux = m->aux;
        float4* own_bnd = m->bnd;
        uint32_t* own_nbr = m->nbr;
        uint32_t* own_cnt = m->nbr_count;
        const int o = 1 - m->cur;
        float4* own_pos = m->pos[o];
        float4* own_vel = m->vel[o];
        int rc = VFS_OK;
        for (int t = 0; t < len && rc == VFS_OK; t++) {
            m->aux = s_aux[t];
            m->bnd = s_bnd[t];
            m->nbr = s_nbr[t];
            m->nbr_count = s_cnt[t];
            m->pos[o] = s_pos[t];
            m->vel[o] = s_vel[t];
            rc = m->enqueue_substep(nullptr);
            if (rc == VFS_OK) {
                const cudaError_t e = cudaMemcpyAsync(s_perm[t], m->sperm, (size_t)m->n * 4,
                                                      cudaMemcpyDeviceToDevice, m->stream);
                if (e != cudaSuccess) rc = fail(VFS_ERR_CUDA, cudaGetErrorString(e));
            }
        }
        m->aux = own_aux;
        m->bnd = own_bnd;
        m->nbr = own_nbr;
        m->nbr_count = own_cnt;
        m->pos[o] = own_pos;
        m->vel[o] = own_vel;
        return rc;
    }

    // Recompute + reverse of one segment of `len` substeps whose input state is in the model.
    int segment_body(int len) {
        int rc = record_segment(len);
        for (int t = len - 1; t >= 0 && rc == VFS_OK; t--) rc = reverse_substep(t);
        return rc;
    }

    // Full segments replay one captured graph; a shorter last segment runs without one.
    int run_segment(int len) {
        if (len != every) return segment_body(len);
        if (!seg_graph) {
            cudaGraph_t g = nullptr;
            VFS_ADJ_TRY(cudaStreamBeginCapture(m->stream, cudaStreamCaptureModeThreadLocal));
            const int rc = segment_body(len);
            const cudaError_t e = cudaStreamEndCapture(m->stream, &g);
            if (rc) {
                if (g) cudaGraphDestroy(g);
                return rc;
            }
            if (e != cudaSuccess) return fail(VFS_ERR_CUDA, std::string("segment capture: ") + cudaGetErrorString(e));
            const cudaError_t ei = cudaGraphInstantiate(&seg_graph, g, 0);
            cudaGraphDestroy(g);
            if (ei != cudaSuccess) {
                seg_graph = nullptr;
                return fail(VFS_ERR_CUDA, std::string("segment graph: ") + cudaGetErrorString(ei));
            }
        }
        VFS_ADJ_TRY(cudaGraphLaunch(seg_graph, m->stream));
        return VFS_OK;
    }

    // One reverse substep: (xbar, vbar) hold the adjoint of the substep's output state; on return
    // they hold the adjoint of its input state.
    int reverse_substep(int t) {
        const uint32_t n = m->n;
        const SceneParams& p = m->scenes[0].params;
        cudaStream_t s = m->stream;
        AdjBuffers B;
        B.pos = s_pos[t];
        B.vel = s_vel[t];
        B.aux = s_aux[t];
        B.bnd = s_bnd[t];
        B.nbr = s_nbr[t];
        B.nbr_count = s_cnt[t];
        B.xbar = xs;
        B.vbar = vs;
        B.abar = abar;
        B.pmbar = pmbar;
        B.pbbar = pbbar;
        B.rhobar = rhobar;
        B.gbar = gbar;
        B.dparams = dparams;
        B.err = m->err;
        const unsigned g256 = (n + 255) / 256;
        k_adj_integrate<<<g256, 256, 0, s>>>(p, n, xbar, vbar, B);
        const unsigned gl = (unsigned)(((size_t)n * kAdjLanes + 127) / 128);
        k_adj_force<kAdjLanes><<<gl, 128, 0, s>>>(p, n, B);
        k_adj_eos<<<g256, 256, 0, s>>>(p, n, B);
        k_adj_density<kAdjLanes><<<gl, 128, 0, s>>>(p, n, B);
        k_adj_unsort<<<g256, 256, 0, s>>>(n, s_perm[t], xs, vs, xbar, vbar);
        VFS_ADJ_TRY(cudaGetLastError());
        return VFS_OK;
    }

    int backward(const float* gx_host, const float* gv_host, float* dv0, float* dx0, double* dpar) {
        if (!forward_done) return fail(VFS_ERR_NOT_READY, "run the rollout forward first");
        const uint32_t n = m->n;
        cudaStream_t s = m->stream;
        const unsigned g256 = (n + 255) / 256;
        VFS_ADJ_TRY(cudaMemsetAsync(dparams, 0, 2 * sizeof(double), s));
        // Seed: by-id gradients of the final state, placed in its (sorted) order.
        for (int which = 0; which < 2; which++) {
            const float* h = which == 0 ? gx_host : gv_host;
            float4* dst = which == 0 ? xbar : vbar;
            if (h) {
                VFS_ADJ_TRY(cudaMemcpyAsync(host_io, h, (size_t)n * 12, cudaMemcpyHostToDevice, s));
                k_adj_by_id<<<g256, 256, 0, s>>>(n, fin_pos, host_io, dst);
            } else {
                VFS_ADJ_TRY(cudaMemsetAsync(dst, 0, (size_t)n * sizeof(float4), s));
            }
        }
        VFS_ADJ_TRY(cudaGetLastError());
        for (int t0 = last_t0(); t0 >= 0; t0 -= every) {
            const int len = t0 + every <= steps ? every : steps - t0;
            int rc = VFS_OK;
            if (t0 == last_t0() && last_recorded) {
                for (int t = len - 1; t >= 0 && rc == VFS_OK; t--) rc = reverse_substep(t);
            } else {
                rc = restore(ck_pos[t0 / every], ck_vel[t0 / every]);
                if (rc == VFS_OK) rc = run_segment(len);
            }
            if (rc) return rc;
        }
        last_recorded = false;  // the records now hold the first segment
        // xbar / vbar now hold the adjoint of the rollout's initial state, in its order.
        if (dv0) {
            k_to_id<<<g256, 256, 0, s>>>(n, ck_pos[0], vbar, host_io);
            VFS_ADJ_TRY(cudaMemcpyAsync(dv0, host_io, (size_t)n * 12, cudaMemcpyDeviceToHost, s));
        }
        if (dx0) {
            k_to_id<<<g256, 256, 0, s>>>(n, ck_pos[0], xbar, host_io);
            VFS_ADJ_TRY(cudaMemcpyAsync(dx0, host_io, (size_t)n * 12, cudaMemcpyDeviceToHost, s));
        }
        double dp[2] = {0.0, 0.0};
        VFS_ADJ_TRY(cudaMemcpyAsync(dp, dparams, sizeof(dp), cudaMemcpyDeviceToHost, s));
        int rc = restore(fin_pos, fin_vel);  // leave the model at the end of the rollout
        if (rc) return rc;
        rc = m->check_device();
        if (rc) {
            uint32_t e = 0;
            cudaMemcpy(&e, m->err, 4, cudaMemcpyDeviceToHost);
            if (e & kErrAdjointOverflow)
                return fail(VFS_ERR_CAPACITY, "a neighbour list exceeded " + std::to_string(cap) +
                                                  " entries: the adjoint needs "
                                              "complete lists");
            return rc;
        }
        if (dpar) {
            dpar[0] = dp[0];
            dpar[1] = dp[1];
        }
        return VFS_OK;
    }
};

}  // namespace vfs

using vfs::fail;

extern "C" {

struct vfs_rollout {
    vfs::Rollout r;
};

int vfs_rollout_create(vfs_model* model, int32_t steps, int32_t checkpoint_every,
                       vfs_rollout** out) {
    vfs::Model* m = vfs_model_impl(model);
    if (!m || !out) return fail(VFS_ERR_INVALID_ARGUMENT, "NULL argument");
    *out = nullptr;
    if (steps < 1) return fail(VFS_ERR_INVALID_ARGUMENT, "steps must be >= 1");
    vfs_rollout* h = new vfs_rollout();
    const int rc = h->r.init(m, steps, checkpoint_every);
    if (rc) {
        delete h;
        return rc;
    }
    *out = h;
    return VFS_OK;
}

int vfs_rollout_destroy(vfs_rollout* r) {
    delete r;
    return VFS_OK;
}

int vfs_rollout_forward(vfs_rollout* r) {
    if (!r) return fail(VFS_ERR_INVALID_ARGUMENT, "NULL rollout");
    return r->r.forward();
}

int vfs_rollout_backward(vfs_rollout* r, const float* dl_dx_final, const float* dl_dv_final,
                         float* dl_dv0, float* dl_dx0, double* dl_dparams) {
    if (!r) return fail(VFS_ERR_INVALID_ARGUMENT, "NULL rollout");
    return r->r.backward(dl_dx_final, dl_dv_final, dl_dv0, dl_dx0, dl_dparams);
}

}  // extern "C"
