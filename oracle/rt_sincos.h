/* rt_sincos.h -- portable binary32 sin/cos of the oracle.
 *
 * TEST INFRASTRUCTURE ONLY: included by oracle/rt_oracle.c and, for the
 * REF_PORTABLE_SINCOS build, by oracle/ref_shim.hpp.  The CUDA kernels carry
 * their own copy of the same operation sequence (csrc/render.cu).
 * GLSL leaves the precision of sin/cos to the implementation
 * (random.glsl:37 uses them); this definition makes host and device agree
 * bit for bit.  Needs <math.h> (rintf) before inclusion.
 */
#ifndef RT_SINCOS_H
#define RT_SINCOS_H
/* Cody-Waite reduction by pi/2 in three binary32 parts, then Taylor
 * polynomials (degree 9 / 10) on [-pi/4, pi/4].  Coefficients are the
 * binary32 roundings of +-1/n!.  Identical operation order in the device code. */
static const float RT_2_OVER_PI = 0x1.45f306p-1f;
static const float RT_PIO2_1 = 0x1.92p+0f;
static const float RT_PIO2_2 = 0x1.fb6p-12f;
static const float RT_PIO2_3 = -0x1.777a5cp-25f;
static const float RT_S1 = -0x1.555556p-3f, RT_S2 = 0x1.111112p-7f, RT_S3 = -0x1.a01a02p-13f,
                   RT_S4 = 0x1.71de3ap-19f;
static const float RT_C1 = -0x1p-1f, RT_C2 = 0x1.555556p-5f, RT_C3 = -0x1.6c16c2p-10f,
                   RT_C4 = 0x1.a01a02p-16f, RT_C5 = -0x1.27e4fcp-22f;

static void rt_sincos(float x, float* s_out, float* c_out) {
  float kf = rintf(x * RT_2_OVER_PI);
  int k = (int)kf;
  float r = x - kf * RT_PIO2_1;
  r = r - kf * RT_PIO2_2;
  r = r - kf * RT_PIO2_3;
  float r2 = r * r;
  float ps = RT_S4;
  ps = ps * r2 + RT_S3;
  ps = ps * r2 + RT_S2;
  ps = ps * r2 + RT_S1;
  float s = r + r * (r2 * ps);
  float pc = RT_C5;
  pc = pc * r2 + RT_C4;
  pc = pc * r2 + RT_C3;
  pc = pc * r2 + RT_C2;
  pc = pc * r2 + RT_C1;
  float c = 1.0f + r2 * pc;
  switch (k & 3) {
    case 0: *s_out = s; *c_out = c; break;
    case 1: *s_out = c; *c_out = -s; break;
    case 2: *s_out = -s; *c_out = -c; break;
    default: *s_out = -c; *c_out = s; break;
  }
}

#endif /* RT_SINCOS_H */
