// gs_train.cu -- the differentiable path's projection backward (the activation of its forward is in
// gs_ply.cu, beside the loader's; the blend backward is in gs_raster.cu).  Gradients carry no
// bit-exactness requirement, so this unit is compiled with FMA contraction.
//
// Forward chain (the reference's formulas, as in gs_ply.cu / gs_cull.cu):
//   parse_ply.comp:62-88   s = exp(log_s), q = quat/|quat| (x, y, z, w), R(q), cov3d = R diag(s^2) R^T,
//                          opacity = sigmoid(logit)
//   projection.comp:95-116 pv = V M pos, Cv = A cov3d A^T (A = V3 M3), J2 = rows (-1/z, 0, x/z^2),
//                          (0, -1/z, y/z^2), cov2d = P2 (J2 Cv J2^T) P2 + diag(1/W^2, 1/H^2)
//   projection.comp:136-174 centre = (P pv).xy / w, colour = max(SH . basis(dir) + 0.5, 0),
//                          dir = normalize(pos - M^-1 eye); the target clamps colour to 1
//   splat.frag              alpha = o exp(-q/2), q = d^T K d, K = cov2d^-1 (= M^T M, M = rot_scale^-1)
// The projection backward takes the per-splat blend gradients of every view (moments of dL/do, colour)
// and applies the chain rule back to the raw parameters, recomputing the forward quantities it needs.
#include "gs_common.cuh"
#include "gs_internal.h"

namespace gs {

__device__ __forceinline__ void quat_rotation(float x, float y, float z, float w, float R[3][3]) {
  const float xx = x * x, yy = y * y, zz = z * z, xy = x * y, xz = x * z, yz = y * z, wx = w * x, wy = w * y,
              wz = w * z;
  R[0][0] = 1.0f - 2.0f * (yy + zz), R[0][1] = 2.0f * (xy - wz), R[0][2] = 2.0f * (xz + wy);
  R[1][0] = 2.0f * (xy + wz), R[1][1] = 1.0f - 2.0f * (xx + zz), R[1][2] = 2.0f * (yz - wx);
  R[2][0] = 2.0f * (xz - wy), R[2][1] = 2.0f * (yz + wx), R[2][2] = 1.0f - 2.0f * (xx + yy);
}

// Degree-3 SH basis B_k(d), the reference's coefficient order (projection.comp:140-163).
__device__ __forceinline__ void sh_basis(float x, float y, float z, float B[16]) {
  const float C0 = 0.28209479177387814f, C1 = 0.4886025119029199f, C20 = 1.0925484305920792f,
              C21 = 0.31539156525252005f, C22 = 0.5462742152960396f, C30 = 0.5900435899266435f,
              C31 = 2.890611442640554f, C32 = 0.4570457994644658f, C33 = 0.3731763325901154f,
              C34 = 1.445305721320277f;
  const float xx = x * x, yy = y * y, zz = z * z, xy = x * y, yz = y * z, xz = x * z;
  B[0] = C0;
  B[1] = -C1 * y;
  B[2] = C1 * z;
  B[3] = -C1 * x;
  B[4] = C20 * xy;
  B[5] = -C20 * yz;
  B[6] = C21 * (2.0f * zz - xx - yy);
  B[7] = -C20 * xz;
  B[8] = C22 * (xx - yy);
  B[9] = -C30 * y * (3.0f * xx - yy);
  B[10] = C31 * xy * z;
  B[11] = -C32 * y * (4.0f * zz - xx - yy);
  B[12] = C33 * z * (2.0f * zz - 3.0f * xx - 3.0f * yy);
  B[13] = -C32 * x * (4.0f * zz - xx - yy);
  B[14] = C34 * z * (xx - yy);
  B[15] = -C30 * x * (xx - 3.0f * yy);
}

// g = sum_k W[k] dB_k/dd: the gradient of the basis contracted with per-coefficient weights, each
// term's partial derivatives written out (no 16 x 3 table is held).
__device__ __forceinline__ void sh_grad_dot(float x, float y, float z, const float W[16], float g[3]) {
  const float C1 = 0.4886025119029199f, C20 = 1.0925484305920792f, C21 = 0.31539156525252005f,
              C22 = 0.5462742152960396f, C30 = 0.5900435899266435f, C31 = 2.890611442640554f,
              C32 = 0.4570457994644658f, C33 = 0.3731763325901154f, C34 = 1.445305721320277f;
  const float xx = x * x, yy = y * y, zz = z * z, xy = x * y, yz = y * z, xz = x * z;
  float gx = -C1 * W[3], gy = -C1 * W[1], gz = C1 * W[2];
  gx += C20 * y * W[4], gy += C20 * x * W[4];
  gy += -C20 * z * W[5], gz += -C20 * y * W[5];
  gx += -2.0f * C21 * x * W[6], gy += -2.0f * C21 * y * W[6], gz += 4.0f * C21 * z * W[6];
  gx += -C20 * z * W[7], gz += -C20 * x * W[7];
  gx += 2.0f * C22 * x * W[8], gy += -2.0f * C22 * y * W[8];
  gx += -6.0f * C30 * xy * W[9], gy += -C30 * (3.0f * xx - 3.0f * yy) * W[9];
  gx += C31 * yz * W[10], gy += C31 * xz * W[10], gz += C31 * xy * W[10];
  gx += 2.0f * C32 * xy * W[11], gy += -C32 * (4.0f * zz - xx - 3.0f * yy) * W[11], gz += -8.0f * C32 * yz * W[11];
  gx += -6.0f * C33 * xz * W[12], gy += -6.0f * C33 * yz * W[12], gz += C33 * (6.0f * zz - 3.0f * xx - 3.0f * yy) * W[12];
  gx += -C32 * (4.0f * zz - 3.0f * xx - yy) * W[13], gy += 2.0f * C32 * xy * W[13], gz += -8.0f * C32 * xz * W[13];
  gx += 2.0f * C34 * xz * W[14], gy += -2.0f * C34 * yz * W[14], gz += C34 * (xx - yy) * W[14];
  gx += -C30 * (3.0f * xx - 3.0f * yy) * W[15], gy += 6.0f * C30 * xy * W[15];
  g[0] = gx, g[1] = gy, g[2] = gz;
}

// m (column-major 4x4) as a row-major 3x3 / 4x4 element
__device__ __forceinline__ float mel(const float* m, int r, int c) { return m[c * 4 + r]; }

constexpr u32 kPbThreads = 128;

// Scale s = exp(log_s), the normalised quaternion, its length and R(q) of splat id (parse_ply.comp:62-88).
__device__ __forceinline__ void scale_rotation(const TrainArgs& a, u32 id, float sc[3], float qn[4], float& qlen,
                                               float R[3][3]) {
  sc[0] = expf(a.log_scales[3 * id]), sc[1] = expf(a.log_scales[3 * id + 1]), sc[2] = expf(a.log_scales[3 * id + 2]);
  const float4 q4 = reinterpret_cast<const float4*>(a.quats)[id];
  qlen = sqrtf(((q4.x * q4.x + q4.y * q4.y) + q4.z * q4.z) + q4.w * q4.w);
  qn[0] = q4.x / qlen, qn[1] = q4.y / qlen, qn[2] = q4.z / qlen, qn[3] = q4.w / qlen;
  quat_rotation(qn[0], qn[1], qn[2], qn[3], R);
}

// Projection backward over every view of one step: a thread per splat walks the views whose blend
// backward reached the splat and accumulates the raw-parameter gradients in registers (SH in shared
// memory), then adds them to the caller's buffers once -- the splat's parameters are read once and no
// atomics are needed however many views there are.  The final maps (quaternion normalisation, exp of
// the log-scales, sigmoid of the logit) are linear in the accumulated gradients, so they are applied
// after the sum over views.
// 4 CTAs per SM: 128 registers, no spills (168 without the bound, 3 CTAs per SM)
__global__ __launch_bounds__(kPbThreads, 4) void k_project_backward(const TrainViews vs, const TrainArgs a) {
  __shared__ float s_gsh[48][kPbThreads];
  const u32 tid = threadIdx.x;
  const u32 stride = gridDim.x * blockDim.x;
  for (u32 id = blockIdx.x * blockDim.x + tid; id < a.n; id += stride) {
    bool ready = false;  // forward quantities of the splat computed (on the first view that needs them)
    float Sg[3][3], o = 0.0f, pos[3];
    // dL/dcov3d summed over the views: cov3d does not depend on the view, so its chain back to scale and
    // rotation runs once per splat, after the view loop
    float gSum[3][3] = {{0.0f, 0.0f, 0.0f}, {0.0f, 0.0f, 0.0f}, {0.0f, 0.0f, 0.0f}};
    float gpos[3] = {0.0f, 0.0f, 0.0f}, g_o = 0.0f;
    const float4* __restrict__ shp = reinterpret_cast<const float4*>(a.sh + 48 * (size_t)id);
#pragma unroll 1
    for (u32 v = 0; v < vs.count; ++v) {
      float gr[12];
      const float4* __restrict__ g4 = reinterpret_cast<const float4*>(vs.grad_rec[v] + (size_t)id * kGradRec);
      bool any = false;
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        const float4 q = __ldg(g4 + k);
        gr[4 * k] = q.x, gr[4 * k + 1] = q.y, gr[4 * k + 2] = q.z, gr[4 * k + 3] = q.w;
      }
#pragma unroll
      for (int k = 0; k < 9; ++k) any |= gr[k] != 0.0f;
      if (!any) continue;  // not in any tile list of this view
      if (!ready) {        // ---- activation (parse_ply.comp:62-88)
        ready = true;
        for (int k = 0; k < 48; ++k) s_gsh[k][tid] = 0.0f;
        float sc[3], qn[4], qlen, R[3][3];
        scale_rotation(a, id, sc, qn, qlen, R);
#pragma unroll
        for (int r = 0; r < 3; ++r)
#pragma unroll
          for (int c = 0; c < 3; ++c)
            Sg[r][c] = R[r][0] * sc[0] * sc[0] * R[c][0] + R[r][1] * sc[1] * sc[1] * R[c][1] +
                       R[r][2] * sc[2] * sc[2] * R[c][2];
        o = 1.0f / (1.0f + expf(-a.opacity_logits[id]));
        pos[0] = a.means[3 * id], pos[1] = a.means[3 * id + 1], pos[2] = a.means[3 * id + 2];
      }
      const FrameConst& fc = vs.fc[v];
      const float* vm = vs.vm[v];  // V M, row-major; its 3 x 3 block is A = V3 M3
      // ---- forward quantities of this view (projection.comp:95-137)
      const auto A = [&](int r, int c) { return vm[4 * r + c]; };
      float pv[4];
#pragma unroll
      for (int r = 0; r < 4; ++r)
        pv[r] = vm[4 * r + 0] * pos[0] + vm[4 * r + 1] * pos[1] + vm[4 * r + 2] * pos[2] + vm[4 * r + 3];
      float Cv[3][3], T3[3][3];
#pragma unroll
      for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c) T3[r][c] = A(r, 0) * Sg[0][c] + A(r, 1) * Sg[1][c] + A(r, 2) * Sg[2][c];
#pragma unroll
      for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c) Cv[r][c] = T3[r][0] * A(c, 0) + T3[r][1] * A(c, 1) + T3[r][2] * A(c, 2);
      const float x = pv[0], y = pv[1], z = pv[2];
      const float J[2][3] = {{-1.0f / z, 0.0f, x / z / z}, {0.0f, -1.0f / z, y / z / z}};
      float JC[2][3], C2[2][2];
#pragma unroll
      for (int r = 0; r < 2; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c) JC[r][c] = J[r][0] * Cv[0][c] + J[r][1] * Cv[1][c] + J[r][2] * Cv[2][c];
#pragma unroll
      for (int r = 0; r < 2; ++r)
#pragma unroll
        for (int c = 0; c < 2; ++c) C2[r][c] = JC[r][0] * J[c][0] + JC[r][1] * J[c][1] + JC[r][2] * J[c][2];
      const float P2[2][2] = {{mel(fc.proj, 0, 0), mel(fc.proj, 0, 1)}, {mel(fc.proj, 1, 0), mel(fc.proj, 1, 1)}};
      float PC[2][2], S2[2][2];
#pragma unroll
      for (int r = 0; r < 2; ++r)
#pragma unroll
        for (int c = 0; c < 2; ++c) PC[r][c] = P2[r][0] * C2[0][c] + P2[r][1] * C2[1][c];
#pragma unroll
      for (int r = 0; r < 2; ++r)
#pragma unroll
        for (int c = 0; c < 2; ++c) S2[r][c] = PC[r][0] * P2[0][c] + PC[r][1] * P2[1][c];
      S2[0][0] += fc.lpx;
      S2[1][1] += fc.lpy;
      const float sa = S2[0][0], sb = S2[1][1], scc = 0.5f * (S2[0][1] + S2[1][0]);
      const float det = sa * sb - scc * scc;
      const float K[2][2] = {{sb / det, -scc / det}, {-scc / det, sa / det}};
      // the blend's moments -> centre and conic gradients (K and o are constant over the splat's pixels)
      const float g_cx = o * (K[0][0] * gr[1] + K[0][1] * gr[2]), g_cy = o * (K[1][0] * gr[1] + K[1][1] * gr[2]);
      const float g_kxx = -0.5f * o * gr[3], g_kyy = -0.5f * o * gr[4], g_kxy2 = -o * gr[5];  // Kxy counted twice
      g_o += gr[0];
      float pc[4];
#pragma unroll
      for (int r = 0; r < 4; ++r)
        pc[r] = mel(fc.proj, r, 0) * pv[0] + mel(fc.proj, r, 1) * pv[1] + mel(fc.proj, r, 2) * pv[2] +
                mel(fc.proj, r, 3) * pv[3];
      const float nx = pc[0] / pc[3], ny = pc[1] / pc[3];
      const float dv[3] = {pos[0] - fc.cam_m[0], pos[1] - fc.cam_m[1], pos[2] - fc.cam_m[2]};
      const float dl = sqrtf(dv[0] * dv[0] + dv[1] * dv[1] + dv[2] * dv[2]);
      const float dir[3] = {dv[0] / dl, dv[1] / dl, dv[2] / dl};
      float B[16];
      sh_basis(dir[0], dir[1], dir[2], B);

      // ---- colour -> SH and view direction (one channel's 16 coefficients at a time); the direction
      // gradient sum_ch gc_ch sum_k c_ch,k dB_k is taken once from the weights W_k = sum_ch gc_ch c_ch,k
      float W[16];
#pragma unroll
      for (int k = 0; k < 16; ++k) W[k] = 0.0f;
#pragma unroll
      for (int ch = 0; ch < 3; ++ch) {
        float c16[16];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          const float4 q = __ldg(shp + 4 * ch + k);
          c16[4 * k] = q.x, c16[4 * k + 1] = q.y, c16[4 * k + 2] = q.z, c16[4 * k + 3] = q.w;
        }
        float col = 0.5f;
#pragma unroll
        for (int k = 0; k < 16; ++k) col += B[k] * c16[k];
        const float gc = (col > 0.0f && col < 1.0f) ? gr[6 + ch] : 0.0f;  // max(., 0) and the target's clamp
        if (gc == 0.0f) continue;
#pragma unroll
        for (int k = 0; k < 16; ++k) {
          s_gsh[16 * ch + k][tid] += B[k] * gc;
          W[k] += c16[k] * gc;
        }
      }
      float gdir[3];
      sh_grad_dot(dir[0], dir[1], dir[2], W, gdir);
      const float dd = dir[0] * gdir[0] + dir[1] * gdir[1] + dir[2] * gdir[2];
      float gp[3] = {(gdir[0] - dir[0] * dd) / dl, (gdir[1] - dir[1] * dd) / dl, (gdir[2] - dir[2] * dd) / dl};

      // ---- conic -> cov2d -> C2 -> (J, Cv) -> cov3d
      const float Gb[2][2] = {{g_kxx, 0.5f * g_kxy2}, {0.5f * g_kxy2, g_kyy}};
      float KG[2][2], gS2[2][2];
#pragma unroll
      for (int r = 0; r < 2; ++r)
#pragma unroll
        for (int c = 0; c < 2; ++c) KG[r][c] = K[r][0] * Gb[0][c] + K[r][1] * Gb[1][c];
#pragma unroll
      for (int r = 0; r < 2; ++r)
#pragma unroll
        for (int c = 0; c < 2; ++c) gS2[r][c] = -(KG[r][0] * K[0][c] + KG[r][1] * K[1][c]);
      float tP[2][2], gC2[2][2];  // gC2 = P2^T gS2 P2^T
#pragma unroll
      for (int r = 0; r < 2; ++r)
#pragma unroll
        for (int c = 0; c < 2; ++c) tP[r][c] = P2[0][r] * gS2[0][c] + P2[1][r] * gS2[1][c];
#pragma unroll
      for (int r = 0; r < 2; ++r)
#pragma unroll
        for (int c = 0; c < 2; ++c) gC2[r][c] = tP[r][0] * P2[c][0] + tP[r][1] * P2[c][1];
      float gCv[3][3];  // J^T gC2 J
#pragma unroll
      for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c)
          gCv[r][c] = J[0][r] * (gC2[0][0] * J[0][c] + gC2[0][1] * J[1][c]) +
                      J[1][r] * (gC2[1][0] * J[0][c] + gC2[1][1] * J[1][c]);
      float gJ[2][3];  // (gC2 + gC2^T) J Cv
#pragma unroll
      for (int r = 0; r < 2; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          const float s0 = gC2[r][0] + gC2[0][r], s1 = gC2[r][1] + gC2[1][r];
          gJ[r][c] = s0 * JC[0][c] + s1 * JC[1][c];
        }
      const float iz2 = 1.0f / (z * z), iz3 = iz2 / z;
      float gpv[3] = {gJ[0][2] * iz2, gJ[1][2] * iz2,
                      (gJ[0][0] + gJ[1][1]) * iz2 - 2.0f * (x * gJ[0][2] + y * gJ[1][2]) * iz3};
      // centre: (P pv).xy / w
      const float iw = 1.0f / pc[3];
      const float gpc[4] = {g_cx * iw, g_cy * iw, 0.0f, -(g_cx * nx + g_cy * ny) * iw};
#pragma unroll
      for (int c = 0; c < 3; ++c)
        gpv[c] += mel(fc.proj, 0, c) * gpc[0] + mel(fc.proj, 1, c) * gpc[1] + mel(fc.proj, 2, c) * gpc[2] +
                  mel(fc.proj, 3, c) * gpc[3];
      // pv = V M pos: the linear part is A
#pragma unroll
      for (int c = 0; c < 3; ++c) gpos[c] += gp[c] + (A(0, c) * gpv[0] + A(1, c) * gpv[1] + A(2, c) * gpv[2]);
      float gS[3][3];  // A^T gCv A
      float tA[3][3];
#pragma unroll
      for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c) tA[r][c] = A(0, r) * gCv[0][c] + A(1, r) * gCv[1][c] + A(2, r) * gCv[2][c];
#pragma unroll
      for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c) gS[r][c] = tA[r][0] * A(0, c) + tA[r][1] * A(1, c) + tA[r][2] * A(2, c);

#pragma unroll
      for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c) gSum[r][c] += gS[r][c];
    }
    if (!ready) continue;
    // ---- cov3d = (R S)(R S)^T -> scale, rotation -> (unnormalised) quaternion gradient, once for the sum
    // over the views (recomputed here rather than kept live through the view loop)
    float sc[3], qn[4], qlen, R[3][3];
    scale_rotation(a, id, sc, qn, qlen, R);
    float gR[3][3], gsc[3] = {0.0f, 0.0f, 0.0f}, gq[4];
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        // d cov / d M_ri with M = R diag(s): (gS + gS^T) M
        const float gM = (gSum[r][0] + gSum[0][r]) * R[0][i] * sc[i] + (gSum[r][1] + gSum[1][r]) * R[1][i] * sc[i] +
                         (gSum[r][2] + gSum[2][r]) * R[2][i] * sc[i];
        gsc[i] += gM * R[r][i];
        gR[r][i] = gM * sc[i];
      }
    {
      const float qx = qn[0], qy = qn[1], qz = qn[2], qw = qn[3];
      gq[0] = 2.0f * (qy * (gR[0][1] + gR[1][0]) + qz * (gR[0][2] + gR[2][0]) + qw * (gR[2][1] - gR[1][2])) -
              4.0f * qx * (gR[1][1] + gR[2][2]);
      gq[1] = 2.0f * (qx * (gR[0][1] + gR[1][0]) + qw * (gR[0][2] - gR[2][0]) + qz * (gR[1][2] + gR[2][1])) -
              4.0f * qy * (gR[0][0] + gR[2][2]);
      gq[2] = 2.0f * (qw * (gR[1][0] - gR[0][1]) + qx * (gR[0][2] + gR[2][0]) + qy * (gR[1][2] + gR[2][1])) -
              4.0f * qz * (gR[0][0] + gR[1][1]);
      gq[3] = 2.0f * (qz * (gR[1][0] - gR[0][1]) + qy * (gR[0][2] - gR[2][0]) + qx * (gR[2][1] - gR[1][2]));
    }
    // ---- the linear maps back to the raw parameters, added once
    float4* __restrict__ gsh = reinterpret_cast<float4*>(a.g_sh + 48 * (size_t)id);
#pragma unroll
    for (int k = 0; k < 12; ++k) {
      const float4 old = gsh[k];
      gsh[k] = make_float4(old.x + s_gsh[4 * k][tid], old.y + s_gsh[4 * k + 1][tid], old.z + s_gsh[4 * k + 2][tid],
                           old.w + s_gsh[4 * k + 3][tid]);
    }
    const float qd = qn[0] * gq[0] + qn[1] * gq[1] + qn[2] * gq[2] + qn[3] * gq[3];
    float4* gq4 = reinterpret_cast<float4*>(a.g_quats) + id;
    const float4 oq = *gq4;
    *gq4 = make_float4(oq.x + (gq[0] - qn[0] * qd) / qlen, oq.y + (gq[1] - qn[1] * qd) / qlen,
                       oq.z + (gq[2] - qn[2] * qd) / qlen, oq.w + (gq[3] - qn[3] * qd) / qlen);
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      a.g_log_scales[3 * id + i] += gsc[i] * sc[i];
      a.g_means[3 * id + i] += gpos[i];
    }
    a.g_opacity_logits[id] += g_o * o * (1.0f - o);
  }
}

cudaError_t launch_project_backward(const TrainViews& vs, const TrainArgs& a, cudaStream_t stream) {
  if (a.n == 0 || vs.count == 0) return cudaSuccess;
  if (vs.count > kMaxTrainViews) return cudaErrorInvalidValue;
  k_project_backward<<<min((a.n + kPbThreads - 1) / kPbThreads, 65535u), kPbThreads, 0, stream>>>(vs, a);
  return cudaGetLastError();
}

}  // namespace gs
