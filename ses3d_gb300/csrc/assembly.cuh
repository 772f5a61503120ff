// assembly.cuh -- node-level pieces shared by the forward node kernel (kernels.cu) and the
// exact discrete adjoint (adjoint.cu): the deterministic gather of the element-local
// contributions of one global node, and the corner-normalised PML profiles and taper.
#pragma once
#include "kernels.cuh"

namespace ses3d {

// Whether element (i, j, k) lies in the PML: pml elements on both x and y sides and at the
// bottom (the top is a free surface; SOURCE/ses3d_init.f90:586). Outside, every profile is
// zero and the taper one.
__device__ __forceinline__ bool in_pml_element(const Consts &c, int i, int j, int k) {
  return i < c.pml || i >= c.ex - c.pml || j < c.pml || j >= c.ey - c.pml || k >= c.ez - c.pml;
}

// Column gy of a global-node index t = gx + GX gy, by the multiply-shift division the
// constants hold (exact for 32-bit t, GX >= 2).
__device__ __forceinline__ int node_row(const Consts &c, unsigned t) {
  const unsigned hi = __umulhi(t, c.gx_magic);
  return (int)((hi + ((t - hi) >> 1)) >> c.gx_shift);
}

// Sum of the (up to eight) element-local contributions F[e][comp][n] to global node
// (gx, gy, gz) of one event, in the reference loop order (element i, then j, then k
// ascending; ses3d_evolution.f90:286-310). F points at the event's [E][3][125] block.
// Whether a node lies on a y or z element face is the same for a warp of consecutive gx
// (one gy row), so the cases do not diverge; the x face (every fourth gx) is predicated.
// Offsets are one 32-bit term per axis (3 N < 2^32 is checked at create); at most four
// contributions are in flight at a time.
__device__ __forceinline__ void gather_node(const Consts &c, const float *F, int gx, int gy, int gz, float &sx,
                                            float &sy, float &sz) {
  const int i0 = gx == 0 ? 0 : (gx - 1) >> 2, i1 = min(gx >> 2, c.ex - 1);
  const int j0 = gy == 0 ? 0 : (gy - 1) >> 2, j1 = min(gy >> 2, c.ey - 1);
  const int k0 = gz == 0 ? 0 : (gz - 1) >> 2, k1 = min(gz >> 2, c.ez - 1);
  const unsigned sy_ = (unsigned)c.ex * 375u, sz_ = sy_ * (unsigned)c.ey;
  const unsigned q0 = ((unsigned)i0 * 371u + (unsigned)gx) + ((unsigned)j0 * (sy_ - 20u) + 5u * (unsigned)gy) +
                      ((unsigned)k0 * (sz_ - 100u) + 25u * (unsigned)gz);
  const unsigned dx = (unsigned)(i1 - i0) * 371u, dy = (unsigned)(j1 - j0) * (sy_ - 20u),
                 dz = (unsigned)(k1 - k0) * (sz_ - 100u);
  const bool ux = i1 != i0, uy = j1 != j0, uz = k1 != k0;
  sx = 0.f; sy = 0.f; sz = 0.f;
  if (!uy && !uz) {
    const float a0 = F[q0], a1 = F[q0 + 125], a2 = F[q0 + 250];
    float b0 = 0.f, b1 = 0.f, b2 = 0.f;
    if (ux) { b0 = F[q0 + dx]; b1 = F[q0 + dx + 125]; b2 = F[q0 + dx + 250]; }
    sx = 0.f + a0; sy = 0.f + a1; sz = 0.f + a2;
    if (ux) { sx += b0; sy += b1; sz += b2; }
  } else if (!uy || !uz) {  // one of the y / z faces: contributions q0, q0 + d (+ the x pair)
    const unsigned d = uz ? dz : dy;
    const float a0 = F[q0], a1 = F[q0 + 125], a2 = F[q0 + 250];
    const float c0 = F[q0 + d], c1 = F[q0 + d + 125], c2 = F[q0 + d + 250];
    float b0 = 0.f, b1 = 0.f, b2 = 0.f, e0 = 0.f, e1 = 0.f, e2 = 0.f;
    if (ux) {
      b0 = F[q0 + dx]; b1 = F[q0 + dx + 125]; b2 = F[q0 + dx + 250];
      e0 = F[q0 + dx + d]; e1 = F[q0 + dx + d + 125]; e2 = F[q0 + dx + d + 250];
    }
    sx = 0.f + a0; sy = 0.f + a1; sz = 0.f + a2;
    sx += c0; sy += c1; sz += c2;
    if (ux) { sx += b0; sy += b1; sz += b2; sx += e0; sy += e1; sz += e2; }
  } else {  // y and z faces: i0 half (4 contributions), then the i1 half
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      if (h == 1 && !ux) break;
      const unsigned q = q0 + (h ? dx : 0u);
      const float f00 = F[q], f01 = F[q + 125], f02 = F[q + 250];
      const float f10 = F[q + dz], f11 = F[q + dz + 125], f12 = F[q + dz + 250];
      const float f20 = F[q + dy], f21 = F[q + dy + 125], f22 = F[q + dy + 250];
      const float f30 = F[q + dy + dz], f31 = F[q + dy + dz + 125], f32 = F[q + dy + dz + 250];
      if (h == 0) { sx = 0.f + f00; sy = 0.f + f01; sz = 0.f + f02; }
      else { sx += f00; sy += f01; sz += f02; }
      sx += f10; sy += f11; sz += f12;
      sx += f20; sy += f21; sz += f22;
      sx += f30; sy += f31; sz += f32;
    }
  }
}

// Corner-normalised PML profiles and taper of one node from its raw axis profiles
// (ses3d_init.f90:678-686), in IEEE round-to-nearest operations as the reference rounds.
__device__ __forceinline__ void pml_profiles(float pxr, float pyr, float pzr, float &px, float &py, float &pz,
                                             float &prof, float &taper) {
  px = 0.f; py = 0.f; pz = 0.f; prof = 0.f; taper = 1.f;
  const float praw = __fadd_rn(__fadd_rn(pxr, pyr), pzr);
  if (praw != 0.f) {
    const float den = __fadd_rn(1.f, __fdiv_rn(praw, 1.2f));
    pz = __fdiv_rn(__fmul_rn(2.f, pzr), den);
    py = __fdiv_rn(__fmul_rn(2.f, pyr), den);
    px = __fdiv_rn(__fmul_rn(2.f, pxr), den);
    prof = __fadd_rn(__fadd_rn(px, py), pz);
    taper = expf(-__fmul_rn(__fmul_rn(0.1f, prof), prof));
  }
}

}  // namespace ses3d
