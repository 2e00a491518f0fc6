// treelet_dp_unrolled.cuh -- generated by gen_treelet_dp.py; do not edit.
//
// The LBVH+ subset DP (src/cuda/lbvh_plus_builder.cu:119-165) for N = 4..7 treelet leaves
// as straight-line code: subset costs in registers, areas A and best splits P in this
// lane's shared-memory columns (stride 32).  Leaves beyond a treelet's own count are
// never part of its subsets, so a smaller treelet can run a larger N.
#pragma once

namespace bvhgb {

// 4 leaves: 25 split evaluations.
__device__ __forceinline__ void dp_unrolled_4(const float* __restrict__ A, uint8_t* __restrict__ P) {
  const float c1 = 0.0f;
  const float c2 = 0.0f;
  float c3;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c2, c1);
    if (v < b) { b = v; bp = 2u; }
    c3 = __fadd_rn(b, A[3 * 32]);
    P[3 * 32] = (uint8_t)bp;
  }
  const float c4 = 0.0f;
  float c5;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c4, c1);
    if (v < b) { b = v; bp = 4u; }
    c5 = __fadd_rn(b, A[5 * 32]);
    P[5 * 32] = (uint8_t)bp;
  }
  float c6;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c4, c2);
    if (v < b) { b = v; bp = 4u; }
    c6 = __fadd_rn(b, A[6 * 32]);
    P[6 * 32] = (uint8_t)bp;
  }
  float c7;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c2, c5);
    if (v < b) { b = v; bp = 2u; }
    v = __fadd_rn(c4, c3);
    if (v < b) { b = v; bp = 4u; }
    v = __fadd_rn(c6, c1);
    if (v < b) { b = v; bp = 6u; }
    c7 = __fadd_rn(b, A[7 * 32]);
    P[7 * 32] = (uint8_t)bp;
  }
  const float c8 = 0.0f;
  float c9;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c8, c1);
    if (v < b) { b = v; bp = 8u; }
    c9 = __fadd_rn(b, A[9 * 32]);
    P[9 * 32] = (uint8_t)bp;
  }
  float c10;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c8, c2);
    if (v < b) { b = v; bp = 8u; }
    c10 = __fadd_rn(b, A[10 * 32]);
    P[10 * 32] = (uint8_t)bp;
  }
  float c11;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c2, c9);
    if (v < b) { b = v; bp = 2u; }
    v = __fadd_rn(c8, c3);
    if (v < b) { b = v; bp = 8u; }
    v = __fadd_rn(c10, c1);
    if (v < b) { b = v; bp = 10u; }
    c11 = __fadd_rn(b, A[11 * 32]);
    P[11 * 32] = (uint8_t)bp;
  }
  float c12;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c8, c4);
    if (v < b) { b = v; bp = 8u; }
    c12 = __fadd_rn(b, A[12 * 32]);
    P[12 * 32] = (uint8_t)bp;
  }
  float c13;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c4, c9);
    if (v < b) { b = v; bp = 4u; }
    v = __fadd_rn(c8, c5);
    if (v < b) { b = v; bp = 8u; }
    v = __fadd_rn(c12, c1);
    if (v < b) { b = v; bp = 12u; }
    c13 = __fadd_rn(b, A[13 * 32]);
    P[13 * 32] = (uint8_t)bp;
  }
  float c14;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c4, c10);
    if (v < b) { b = v; bp = 4u; }
    v = __fadd_rn(c8, c6);
    if (v < b) { b = v; bp = 8u; }
    v = __fadd_rn(c12, c2);
    if (v < b) { b = v; bp = 12u; }
    c14 = __fadd_rn(b, A[14 * 32]);
    P[14 * 32] = (uint8_t)bp;
  }
  {
    float b = kTlInf, b2 = kTlInf, v, v2;
    uint32_t bp = 0xffu, bp2 = 0xffu;
    v = __fadd_rn(c2, c13);
    if (v < b) { b = v; bp = 2u; }
    v2 = __fadd_rn(c10, c5);
    if (v2 < b2) { b2 = v2; bp2 = 10u; }
    v = __fadd_rn(c4, c11);
    if (v < b) { b = v; bp = 4u; }
    v2 = __fadd_rn(c12, c3);
    if (v2 < b2) { b2 = v2; bp2 = 12u; }
    v = __fadd_rn(c6, c9);
    if (v < b) { b = v; bp = 6u; }
    v2 = __fadd_rn(c14, c1);
    if (v2 < b2) { b2 = v2; bp2 = 14u; }
    v = __fadd_rn(c8, c7);
    if (v < b) { b = v; bp = 8u; }
    if (b2 < b) { b = b2; bp = bp2; }
    P[15 * 32] = (uint8_t)bp;
  }
}

// 5 leaves: 90 split evaluations.
__device__ __forceinline__ void dp_unrolled_5(const float* __restrict__ A, uint8_t* __restrict__ P) {
  const float c1 = 0.0f;
  const float c2 = 0.0f;
  float c3;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c2, c1);
    if (v < b) { b = v; bp = 2u; }
    c3 = __fadd_rn(b, A[3 * 32]);
    P[3 * 32] = (uint8_t)bp;
  }
  const float c4 = 0.0f;
  float c5;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c4, c1);
    if (v < b) { b = v; bp = 4u; }
    c5 = __fadd_rn(b, A[5 * 32]);
    P[5 * 32] = (uint8_t)bp;
  }
  float c6;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c4, c2);
    if (v < b) { b = v; bp = 4u; }
    c6 = __fadd_rn(b, A[6 * 32]);
    P[6 * 32] = (uint8_t)bp;
  }
  float c7;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c2, c5);
    if (v < b) { b = v; bp = 2u; }
    v = __fadd_rn(c4, c3);
    if (v < b) { b = v; bp = 4u; }
    v = __fadd_rn(c6, c1);
    if (v < b) { b = v; bp = 6u; }
    c7 = __fadd_rn(b, A[7 * 32]);
    P[7 * 32] = (uint8_t)bp;
  }
  const float c8 = 0.0f;
  float c9;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c8, c1);
    if (v < b) { b = v; bp = 8u; }
    c9 = __fadd_rn(b, A[9 * 32]);
    P[9 * 32] = (uint8_t)bp;
  }
  float c10;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c8, c2);
    if (v < b) { b = v; bp = 8u; }
    c10 = __fadd_rn(b, A[10 * 32]);
    P[10 * 32] = (uint8_t)bp;
  }
  float c11;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c2, c9);
    if (v < b) { b = v; bp = 2u; }
    v = __fadd_rn(c8, c3);
    if (v < b) { b = v; bp = 8u; }
    v = __fadd_rn(c10, c1);
    if (v < b) { b = v; bp = 10u; }
    c11 = __fadd_rn(b, A[11 * 32]);
    P[11 * 32] = (uint8_t)bp;
  }
  float c12;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c8, c4);
    if (v < b) { b = v; bp = 8u; }
    c12 = __fadd_rn(b, A[12 * 32]);
    P[12 * 32] = (uint8_t)bp;
  }
  float c13;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c4, c9);
    if (v < b) { b = v; bp = 4u; }
    v = __fadd_rn(c8, c5);
    if (v < b) { b = v; bp = 8u; }
    v = __fadd_rn(c12, c1);
    if (v < b) { b = v; bp = 12u; }
    c13 = __fadd_rn(b, A[13 * 32]);
    P[13 * 32] = (uint8_t)bp;
  }
  float c14;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c4, c10);
    if (v < b) { b = v; bp = 4u; }
    v = __fadd_rn(c8, c6);
    if (v < b) { b = v; bp = 8u; }
    v = __fadd_rn(c12, c2);
    if (v < b) { b = v; bp = 12u; }
    c14 = __fadd_rn(b, A[14 * 32]);
    P[14 * 32] = (uint8_t)bp;
  }
  float c15;
  {
    float b = kTlInf, b2 = kTlInf, v, v2;
    uint32_t bp = 0xffu, bp2 = 0xffu;
    v = __fadd_rn(c2, c13);
    if (v < b) { b = v; bp = 2u; }
    v2 = __fadd_rn(c10, c5);
    if (v2 < b2) { b2 = v2; bp2 = 10u; }
    v = __fadd_rn(c4, c11);
    if (v < b) { b = v; bp = 4u; }
    v2 = __fadd_rn(c12, c3);
    if (v2 < b2) { b2 = v2; bp2 = 12u; }
    v = __fadd_rn(c6, c9);
    if (v < b) { b = v; bp = 6u; }
    v2 = __fadd_rn(c14, c1);
    if (v2 < b2) { b2 = v2; bp2 = 14u; }
    v = __fadd_rn(c8, c7);
    if (v < b) { b = v; bp = 8u; }
    if (b2 < b) { b = b2; bp = bp2; }
    c15 = __fadd_rn(b, A[15 * 32]);
    P[15 * 32] = (uint8_t)bp;
  }
  const float c16 = 0.0f;
  float c17;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c16, c1);
    if (v < b) { b = v; bp = 16u; }
    c17 = __fadd_rn(b, A[17 * 32]);
    P[17 * 32] = (uint8_t)bp;
  }
  float c18;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c16, c2);
    if (v < b) { b = v; bp = 16u; }
    c18 = __fadd_rn(b, A[18 * 32]);
    P[18 * 32] = (uint8_t)bp;
  }
  float c19;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c2, c17);
    if (v < b) { b = v; bp = 2u; }
    v = __fadd_rn(c16, c3);
    if (v < b) { b = v; bp = 16u; }
    v = __fadd_rn(c18, c1);
    if (v < b) { b = v; bp = 18u; }
    c19 = __fadd_rn(b, A[19 * 32]);
    P[19 * 32] = (uint8_t)bp;
  }
  float c20;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c16, c4);
    if (v < b) { b = v; bp = 16u; }
    c20 = __fadd_rn(b, A[20 * 32]);
    P[20 * 32] = (uint8_t)bp;
  }
  float c21;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c4, c17);
    if (v < b) { b = v; bp = 4u; }
    v = __fadd_rn(c16, c5);
    if (v < b) { b = v; bp = 16u; }
    v = __fadd_rn(c20, c1);
    if (v < b) { b = v; bp = 20u; }
    c21 = __fadd_rn(b, A[21 * 32]);
    P[21 * 32] = (uint8_t)bp;
  }
  float c22;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c4, c18);
    if (v < b) { b = v; bp = 4u; }
    v = __fadd_rn(c16, c6);
    if (v < b) { b = v; bp = 16u; }
    v = __fadd_rn(c20, c2);
    if (v < b) { b = v; bp = 20u; }
    c22 = __fadd_rn(b, A[22 * 32]);
    P[22 * 32] = (uint8_t)bp;
  }
  float c23;
  {
    float b = kTlInf, b2 = kTlInf, v, v2;
    uint32_t bp = 0xffu, bp2 = 0xffu;
    v = __fadd_rn(c2, c21);
    if (v < b) { b = v; bp = 2u; }
    v2 = __fadd_rn(c18, c5);
    if (v2 < b2) { b2 = v2; bp2 = 18u; }
    v = __fadd_rn(c4, c19);
    if (v < b) { b = v; bp = 4u; }
    v2 = __fadd_rn(c20, c3);
    if (v2 < b2) { b2 = v2; bp2 = 20u; }
    v = __fadd_rn(c6, c17);
    if (v < b) { b = v; bp = 6u; }
    v2 = __fadd_rn(c22, c1);
    if (v2 < b2) { b2 = v2; bp2 = 22u; }
    v = __fadd_rn(c16, c7);
    if (v < b) { b = v; bp = 16u; }
    if (b2 < b) { b = b2; bp = bp2; }
    c23 = __fadd_rn(b, A[23 * 32]);
    P[23 * 32] = (uint8_t)bp;
  }
  float c24;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c16, c8);
    if (v < b) { b = v; bp = 16u; }
    c24 = __fadd_rn(b, A[24 * 32]);
    P[24 * 32] = (uint8_t)bp;
  }
  float c25;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c8, c17);
    if (v < b) { b = v; bp = 8u; }
    v = __fadd_rn(c16, c9);
    if (v < b) { b = v; bp = 16u; }
    v = __fadd_rn(c24, c1);
    if (v < b) { b = v; bp = 24u; }
    c25 = __fadd_rn(b, A[25 * 32]);
    P[25 * 32] = (uint8_t)bp;
  }
  float c26;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c8, c18);
    if (v < b) { b = v; bp = 8u; }
    v = __fadd_rn(c16, c10);
    if (v < b) { b = v; bp = 16u; }
    v = __fadd_rn(c24, c2);
    if (v < b) { b = v; bp = 24u; }
    c26 = __fadd_rn(b, A[26 * 32]);
    P[26 * 32] = (uint8_t)bp;
  }
  float c27;
  {
    float b = kTlInf, b2 = kTlInf, v, v2;
    uint32_t bp = 0xffu, bp2 = 0xffu;
    v = __fadd_rn(c2, c25);
    if (v < b) { b = v; bp = 2u; }
    v2 = __fadd_rn(c18, c9);
    if (v2 < b2) { b2 = v2; bp2 = 18u; }
    v = __fadd_rn(c8, c19);
    if (v < b) { b = v; bp = 8u; }
    v2 = __fadd_rn(c24, c3);
    if (v2 < b2) { b2 = v2; bp2 = 24u; }
    v = __fadd_rn(c10, c17);
    if (v < b) { b = v; bp = 10u; }
    v2 = __fadd_rn(c26, c1);
    if (v2 < b2) { b2 = v2; bp2 = 26u; }
    v = __fadd_rn(c16, c11);
    if (v < b) { b = v; bp = 16u; }
    if (b2 < b) { b = b2; bp = bp2; }
    c27 = __fadd_rn(b, A[27 * 32]);
    P[27 * 32] = (uint8_t)bp;
  }
  float c28;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c8, c20);
    if (v < b) { b = v; bp = 8u; }
    v = __fadd_rn(c16, c12);
    if (v < b) { b = v; bp = 16u; }
    v = __fadd_rn(c24, c4);
    if (v < b) { b = v; bp = 24u; }
    c28 = __fadd_rn(b, A[28 * 32]);
    P[28 * 32] = (uint8_t)bp;
  }
  float c29;
  {
    float b = kTlInf, b2 = kTlInf, v, v2;
    uint32_t bp = 0xffu, bp2 = 0xffu;
    v = __fadd_rn(c4, c25);
    if (v < b) { b = v; bp = 4u; }
    v2 = __fadd_rn(c20, c9);
    if (v2 < b2) { b2 = v2; bp2 = 20u; }
    v = __fadd_rn(c8, c21);
    if (v < b) { b = v; bp = 8u; }
    v2 = __fadd_rn(c24, c5);
    if (v2 < b2) { b2 = v2; bp2 = 24u; }
    v = __fadd_rn(c12, c17);
    if (v < b) { b = v; bp = 12u; }
    v2 = __fadd_rn(c28, c1);
    if (v2 < b2) { b2 = v2; bp2 = 28u; }
    v = __fadd_rn(c16, c13);
    if (v < b) { b = v; bp = 16u; }
    if (b2 < b) { b = b2; bp = bp2; }
    c29 = __fadd_rn(b, A[29 * 32]);
    P[29 * 32] = (uint8_t)bp;
  }
  float c30;
  {
    float b = kTlInf, b2 = kTlInf, v, v2;
    uint32_t bp = 0xffu, bp2 = 0xffu;
    v = __fadd_rn(c4, c26);
    if (v < b) { b = v; bp = 4u; }
    v2 = __fadd_rn(c20, c10);
    if (v2 < b2) { b2 = v2; bp2 = 20u; }
    v = __fadd_rn(c8, c22);
    if (v < b) { b = v; bp = 8u; }
    v2 = __fadd_rn(c24, c6);
    if (v2 < b2) { b2 = v2; bp2 = 24u; }
    v = __fadd_rn(c12, c18);
    if (v < b) { b = v; bp = 12u; }
    v2 = __fadd_rn(c28, c2);
    if (v2 < b2) { b2 = v2; bp2 = 28u; }
    v = __fadd_rn(c16, c14);
    if (v < b) { b = v; bp = 16u; }
    if (b2 < b) { b = b2; bp = bp2; }
    c30 = __fadd_rn(b, A[30 * 32]);
    P[30 * 32] = (uint8_t)bp;
  }
  {
    float b = kTlInf, b2 = kTlInf, v, v2;
    uint32_t bp = 0xffu, bp2 = 0xffu;
    v = __fadd_rn(c2, c29);
    if (v < b) { b = v; bp = 2u; }
    v2 = __fadd_rn(c18, c13);
    if (v2 < b2) { b2 = v2; bp2 = 18u; }
    v = __fadd_rn(c4, c27);
    if (v < b) { b = v; bp = 4u; }
    v2 = __fadd_rn(c20, c11);
    if (v2 < b2) { b2 = v2; bp2 = 20u; }
    v = __fadd_rn(c6, c25);
    if (v < b) { b = v; bp = 6u; }
    v2 = __fadd_rn(c22, c9);
    if (v2 < b2) { b2 = v2; bp2 = 22u; }
    v = __fadd_rn(c8, c23);
    if (v < b) { b = v; bp = 8u; }
    v2 = __fadd_rn(c24, c7);
    if (v2 < b2) { b2 = v2; bp2 = 24u; }
    v = __fadd_rn(c10, c21);
    if (v < b) { b = v; bp = 10u; }
    v2 = __fadd_rn(c26, c5);
    if (v2 < b2) { b2 = v2; bp2 = 26u; }
    v = __fadd_rn(c12, c19);
    if (v < b) { b = v; bp = 12u; }
    v2 = __fadd_rn(c28, c3);
    if (v2 < b2) { b2 = v2; bp2 = 28u; }
    v = __fadd_rn(c14, c17);
    if (v < b) { b = v; bp = 14u; }
    v2 = __fadd_rn(c30, c1);
    if (v2 < b2) { b2 = v2; bp2 = 30u; }
    v = __fadd_rn(c16, c15);
    if (v < b) { b = v; bp = 16u; }
    if (b2 < b) { b = b2; bp = bp2; }
    P[31 * 32] = (uint8_t)bp;
  }
}

// 6 leaves: 301 split evaluations.
__device__ __forceinline__ void dp_unrolled_6(const float* __restrict__ A, uint8_t* __restrict__ P) {
  const float c1 = 0.0f;
  const float c2 = 0.0f;
  float c3;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c2, c1);
    if (v < b) { b = v; bp = 2u; }
    c3 = __fadd_rn(b, A[3 * 32]);
    P[3 * 32] = (uint8_t)bp;
  }
  const float c4 = 0.0f;
  float c5;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c4, c1);
    if (v < b) { b = v; bp = 4u; }
    c5 = __fadd_rn(b, A[5 * 32]);
    P[5 * 32] = (uint8_t)bp;
  }
  float c6;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c4, c2);
    if (v < b) { b = v; bp = 4u; }
    c6 = __fadd_rn(b, A[6 * 32]);
    P[6 * 32] = (uint8_t)bp;
  }
  float c7;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c2, c5);
    if (v < b) { b = v; bp = 2u; }
    v = __fadd_rn(c4, c3);
    if (v < b) { b = v; bp = 4u; }
    v = __fadd_rn(c6, c1);
    if (v < b) { b = v; bp = 6u; }
    c7 = __fadd_rn(b, A[7 * 32]);
    P[7 * 32] = (uint8_t)bp;
  }
  const float c8 = 0.0f;
  float c9;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c8, c1);
    if (v < b) { b = v; bp = 8u; }
    c9 = __fadd_rn(b, A[9 * 32]);
    P[9 * 32] = (uint8_t)bp;
  }
  float c10;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c8, c2);
    if (v < b) { b = v; bp = 8u; }
    c10 = __fadd_rn(b, A[10 * 32]);
    P[10 * 32] = (uint8_t)bp;
  }
  float c11;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c2, c9);
    if (v < b) { b = v; bp = 2u; }
    v = __fadd_rn(c8, c3);
    if (v < b) { b = v; bp = 8u; }
    v = __fadd_rn(c10, c1);
    if (v < b) { b = v; bp = 10u; }
    c11 = __fadd_rn(b, A[11 * 32]);
    P[11 * 32] = (uint8_t)bp;
  }
  float c12;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c8, c4);
    if (v < b) { b = v; bp = 8u; }
    c12 = __fadd_rn(b, A[12 * 32]);
    P[12 * 32] = (uint8_t)bp;
  }
  float c13;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c4, c9);
    if (v < b) { b = v; bp = 4u; }
    v = __fadd_rn(c8, c5);
    if (v < b) { b = v; bp = 8u; }
    v = __fadd_rn(c12, c1);
    if (v < b) { b = v; bp = 12u; }
    c13 = __fadd_rn(b, A[13 * 32]);
    P[13 * 32] = (uint8_t)bp;
  }
  float c14;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c4, c10);
    if (v < b) { b = v; bp = 4u; }
    v = __fadd_rn(c8, c6);
    if (v < b) { b = v; bp = 8u; }
    v = __fadd_rn(c12, c2);
    if (v < b) { b = v; bp = 12u; }
    c14 = __fadd_rn(b, A[14 * 32]);
    P[14 * 32] = (uint8_t)bp;
  }
  float c15;
  {
    float b = kTlInf, b2 = kTlInf, v, v2;
    uint32_t bp = 0xffu, bp2 = 0xffu;
    v = __fadd_rn(c2, c13);
    if (v < b) { b = v; bp = 2u; }
    v2 = __fadd_rn(c10, c5);
    if (v2 < b2) { b2 = v2; bp2 = 10u; }
    v = __fadd_rn(c4, c11);
    if (v < b) { b = v; bp = 4u; }
    v2 = __fadd_rn(c12, c3);
    if (v2 < b2) { b2 = v2; bp2 = 12u; }
    v = __fadd_rn(c6, c9);
    if (v < b) { b = v; bp = 6u; }
    v2 = __fadd_rn(c14, c1);
    if (v2 < b2) { b2 = v2; bp2 = 14u; }
    v = __fadd_rn(c8, c7);
    if (v < b) { b = v; bp = 8u; }
    if (b2 < b) { b = b2; bp = bp2; }
    c15 = __fadd_rn(b, A[15 * 32]);
    P[15 * 32] = (uint8_t)bp;
  }
  const float c16 = 0.0f;
  float c17;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c16, c1);
    if (v < b) { b = v; bp = 16u; }
    c17 = __fadd_rn(b, A[17 * 32]);
    P[17 * 32] = (uint8_t)bp;
  }
  float c18;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c16, c2);
    if (v < b) { b = v; bp = 16u; }
    c18 = __fadd_rn(b, A[18 * 32]);
    P[18 * 32] = (uint8_t)bp;
  }
  float c19;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c2, c17);
    if (v < b) { b = v; bp = 2u; }
    v = __fadd_rn(c16, c3);
    if (v < b) { b = v; bp = 16u; }
    v = __fadd_rn(c18, c1);
    if (v < b) { b = v; bp = 18u; }
    c19 = __fadd_rn(b, A[19 * 32]);
    P[19 * 32] = (uint8_t)bp;
  }
  float c20;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c16, c4);
    if (v < b) { b = v; bp = 16u; }
    c20 = __fadd_rn(b, A[20 * 32]);
    P[20 * 32] = (uint8_t)bp;
  }
  float c21;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c4, c17);
    if (v < b) { b = v; bp = 4u; }
    v = __fadd_rn(c16, c5);
    if (v < b) { b = v; bp = 16u; }
    v = __fadd_rn(c20, c1);
    if (v < b) { b = v; bp = 20u; }
    c21 = __fadd_rn(b, A[21 * 32]);
    P[21 * 32] = (uint8_t)bp;
  }
  float c22;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c4, c18);
    if (v < b) { b = v; bp = 4u; }
    v = __fadd_rn(c16, c6);
    if (v < b) { b = v; bp = 16u; }
    v = __fadd_rn(c20, c2);
    if (v < b) { b = v; bp = 20u; }
    c22 = __fadd_rn(b, A[22 * 32]);
    P[22 * 32] = (uint8_t)bp;
  }
  float c23;
  {
    float b = kTlInf, b2 = kTlInf, v, v2;
    uint32_t bp = 0xffu, bp2 = 0xffu;
    v = __fadd_rn(c2, c21);
    if (v < b) { b = v; bp = 2u; }
    v2 = __fadd_rn(c18, c5);
    if (v2 < b2) { b2 = v2; bp2 = 18u; }
    v = __fadd_rn(c4, c19);
    if (v < b) { b = v; bp = 4u; }
    v2 = __fadd_rn(c20, c3);
    if (v2 < b2) { b2 = v2; bp2 = 20u; }
    v = __fadd_rn(c6, c17);
    if (v < b) { b = v; bp = 6u; }
    v2 = __fadd_rn(c22, c1);
    if (v2 < b2) { b2 = v2; bp2 = 22u; }
    v = __fadd_rn(c16, c7);
    if (v < b) { b = v; bp = 16u; }
    if (b2 < b) { b = b2; bp = bp2; }
    c23 = __fadd_rn(b, A[23 * 32]);
    P[23 * 32] = (uint8_t)bp;
  }
  float c24;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c16, c8);
    if (v < b) { b = v; bp = 16u; }
    c24 = __fadd_rn(b, A[24 * 32]);
    P[24 * 32] = (uint8_t)bp;
  }
  float c25;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c8, c17);
    if (v < b) { b = v; bp = 8u; }
    v = __fadd_rn(c16, c9);
    if (v < b) { b = v; bp = 16u; }
    v = __fadd_rn(c24, c1);
    if (v < b) { b = v; bp = 24u; }
    c25 = __fadd_rn(b, A[25 * 32]);
    P[25 * 32] = (uint8_t)bp;
  }
  float c26;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c8, c18);
    if (v < b) { b = v; bp = 8u; }
    v = __fadd_rn(c16, c10);
    if (v < b) { b = v; bp = 16u; }
    v = __fadd_rn(c24, c2);
    if (v < b) { b = v; bp = 24u; }
    c26 = __fadd_rn(b, A[26 * 32]);
    P[26 * 32] = (uint8_t)bp;
  }
  float c27;
  {
    float b = kTlInf, b2 = kTlInf, v, v2;
    uint32_t bp = 0xffu, bp2 = 0xffu;
    v = __fadd_rn(c2, c25);
    if (v < b) { b = v; bp = 2u; }
    v2 = __fadd_rn(c18, c9);
    if (v2 < b2) { b2 = v2; bp2 = 18u; }
    v = __fadd_rn(c8, c19);
    if (v < b) { b = v; bp = 8u; }
    v2 = __fadd_rn(c24, c3);
    if (v2 < b2) { b2 = v2; bp2 = 24u; }
    v = __fadd_rn(c10, c17);
    if (v < b) { b = v; bp = 10u; }
    v2 = __fadd_rn(c26, c1);
    if (v2 < b2) { b2 = v2; bp2 = 26u; }
    v = __fadd_rn(c16, c11);
    if (v < b) { b = v; bp = 16u; }
    if (b2 < b) { b = b2; bp = bp2; }
    c27 = __fadd_rn(b, A[27 * 32]);
    P[27 * 32] = (uint8_t)bp;
  }
  float c28;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c8, c20);
    if (v < b) { b = v; bp = 8u; }
    v = __fadd_rn(c16, c12);
    if (v < b) { b = v; bp = 16u; }
    v = __fadd_rn(c24, c4);
    if (v < b) { b = v; bp = 24u; }
    c28 = __fadd_rn(b, A[28 * 32]);
    P[28 * 32] = (uint8_t)bp;
  }
  float c29;
  {
    float b = kTlInf, b2 = kTlInf, v, v2;
    uint32_t bp = 0xffu, bp2 = 0xffu;
    v = __fadd_rn(c4, c25);
    if (v < b) { b = v; bp = 4u; }
    v2 = __fadd_rn(c20, c9);
    if (v2 < b2) { b2 = v2; bp2 = 20u; }
    v = __fadd_rn(c8, c21);
    if (v < b) { b = v; bp = 8u; }
    v2 = __fadd_rn(c24, c5);
    if (v2 < b2) { b2 = v2; bp2 = 24u; }
    v = __fadd_rn(c12, c17);
    if (v < b) { b = v; bp = 12u; }
    v2 = __fadd_rn(c28, c1);
    if (v2 < b2) { b2 = v2; bp2 = 28u; }
    v = __fadd_rn(c16, c13);
    if (v < b) { b = v; bp = 16u; }
    if (b2 < b) { b = b2; bp = bp2; }
    c29 = __fadd_rn(b, A[29 * 32]);
    P[29 * 32] = (uint8_t)bp;
  }
  float c30;
  {
    float b = kTlInf, b2 = kTlInf, v, v2;
    uint32_t bp = 0xffu, bp2 = 0xffu;
    v = __fadd_rn(c4, c26);
    if (v < b) { b = v; bp = 4u; }
    v2 = __fadd_rn(c20, c10);
    if (v2 < b2) { b2 = v2; bp2 = 20u; }
    v = __fadd_rn(c8, c22);
    if (v < b) { b = v; bp = 8u; }
    v2 = __fadd_rn(c24, c6);
    if (v2 < b2) { b2 = v2; bp2 = 24u; }
    v = __fadd_rn(c12, c18);
    if (v < b) { b = v; bp = 12u; }
    v2 = __fadd_rn(c28, c2);
    if (v2 < b2) { b2 = v2; bp2 = 28u; }
    v = __fadd_rn(c16, c14);
    if (v < b) { b = v; bp = 16u; }
    if (b2 < b) { b = b2; bp = bp2; }
    c30 = __fadd_rn(b, A[30 * 32]);
    P[30 * 32] = (uint8_t)bp;
  }
  float c31;
  {
    float b = kTlInf, b2 = kTlInf, v, v2;
    uint32_t bp = 0xffu, bp2 = 0xffu;
    v = __fadd_rn(c2, c29);
    if (v < b) { b = v; bp = 2u; }
    v2 = __fadd_rn(c18, c13);
    if (v2 < b2) { b2 = v2; bp2 = 18u; }
    v = __fadd_rn(c4, c27);
    if (v < b) { b = v; bp = 4u; }
    v2 = __fadd_rn(c20, c11);
    if (v2 < b2) { b2 = v2; bp2 = 20u; }
    v = __fadd_rn(c6, c25);
    if (v < b) { b = v; bp = 6u; }
    v2 = __fadd_rn(c22, c9);
    if (v2 < b2) { b2 = v2; bp2 = 22u; }
    v = __fadd_rn(c8, c23);
    if (v < b) { b = v; bp = 8u; }
    v2 = __fadd_rn(c24, c7);
    if (v2 < b2) { b2 = v2; bp2 = 24u; }
    v = __fadd_rn(c10, c21);
    if (v < b) { b = v; bp = 10u; }
    v2 = __fadd_rn(c26, c5);
    if (v2 < b2) { b2 = v2; bp2 = 26u; }
    v = __fadd_rn(c12, c19);
    if (v < b) { b = v; bp = 12u; }
    v2 = __fadd_rn(c28, c3);
    if (v2 < b2) { b2 = v2; bp2 = 28u; }
    v = __fadd_rn(c14, c17);
    if (v < b) { b = v; bp = 14u; }
    v2 = __fadd_rn(c30, c1);
    if (v2 < b2) { b2 = v2; bp2 = 30u; }
    v = __fadd_rn(c16, c15);
    if (v < b) { b = v; bp = 16u; }
    if (b2 < b) { b = b2; bp = bp2; }
    c31 = __fadd_rn(b, A[31 * 32]);
    P[31 * 32] = (uint8_t)bp;
  }
  const float c32 = 0.0f;
  float c33;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c32, c1);
    if (v < b) { b = v; bp = 32u; }
    c33 = __fadd_rn(b, A[33 * 32]);
    P[33 * 32] = (uint8_t)bp;
  }
  float c34;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c32, c2);
    if (v < b) { b = v; bp = 32u; }
    c34 = __fadd_rn(b, A[34 * 32]);
    P[34 * 32] = (uint8_t)bp;
  }
  float c35;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c2, c33);
    if (v < b) { b = v; bp = 2u; }
    v = __fadd_rn(c32, c3);
    if (v < b) { b = v; bp = 32u; }
    v = __fadd_rn(c34, c1);
    if (v < b) { b = v; bp = 34u; }
    c35 = __fadd_rn(b, A[35 * 32]);
    P[35 * 32] = (uint8_t)bp;
  }
  float c36;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c32, c4);
    if (v < b) { b = v; bp = 32u; }
    c36 = __fadd_rn(b, A[36 * 32]);
    P[36 * 32] = (uint8_t)bp;
  }
  float c37;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c4, c33);
    if (v < b) { b = v; bp = 4u; }
    v = __fadd_rn(c32, c5);
    if (v < b) { b = v; bp = 32u; }
    v = __fadd_rn(c36, c1);
    if (v < b) { b = v; bp = 36u; }
    c37 = __fadd_rn(b, A[37 * 32]);
    P[37 * 32] = (uint8_t)bp;
  }
  float c38;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c4, c34);
    if (v < b) { b = v; bp = 4u; }
    v = __fadd_rn(c32, c6);
    if (v < b) { b = v; bp = 32u; }
    v = __fadd_rn(c36, c2);
    if (v < b) { b = v; bp = 36u; }
    c38 = __fadd_rn(b, A[38 * 32]);
    P[38 * 32] = (uint8_t)bp;
  }
  float c39;
  {
    float b = kTlInf, b2 = kTlInf, v, v2;
    uint32_t bp = 0xffu, bp2 = 0xffu;
    v = __fadd_rn(c2, c37);
    if (v < b) { b = v; bp = 2u; }
    v2 = __fadd_rn(c34, c5);
    if (v2 < b2) { b2 = v2; bp2 = 34u; }
    v = __fadd_rn(c4, c35);
    if (v < b) { b = v; bp = 4u; }
    v2 = __fadd_rn(c36, c3);
    if (v2 < b2) { b2 = v2; bp2 = 36u; }
    v = __fadd_rn(c6, c33);
    if (v < b) { b = v; bp = 6u; }
    v2 = __fadd_rn(c38, c1);
    if (v2 < b2) { b2 = v2; bp2 = 38u; }
    v = __fadd_rn(c32, c7);
    if (v < b) { b = v; bp = 32u; }
    if (b2 < b) { b = b2; bp = bp2; }
    c39 = __fadd_rn(b, A[39 * 32]);
    P[39 * 32] = (uint8_t)bp;
  }
  float c40;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c32, c8);
    if (v < b) { b = v; bp = 32u; }
    c40 = __fadd_rn(b, A[40 * 32]);
    P[40 * 32] = (uint8_t)bp;
  }
  float c41;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c8, c33);
    if (v < b) { b = v; bp = 8u; }
    v = __fadd_rn(c32, c9);
    if (v < b) { b = v; bp = 32u; }
    v = __fadd_rn(c40, c1);
    if (v < b) { b = v; bp = 40u; }
    c41 = __fadd_rn(b, A[41 * 32]);
    P[41 * 32] = (uint8_t)bp;
  }
  float c42;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c8, c34);
    if (v < b) { b = v; bp = 8u; }
    v = __fadd_rn(c32, c10);
    if (v < b) { b = v; bp = 32u; }
    v = __fadd_rn(c40, c2);
    if (v < b) { b = v; bp = 40u; }
    c42 = __fadd_rn(b, A[42 * 32]);
    P[42 * 32] = (uint8_t)bp;
  }
  float c43;
  {
    float b = kTlInf, b2 = kTlInf, v, v2;
    uint32_t bp = 0xffu, bp2 = 0xffu;
    v = __fadd_rn(c2, c41);
    if (v < b) { b = v; bp = 2u; }
    v2 = __fadd_rn(c34, c9);
    if (v2 < b2) { b2 = v2; bp2 = 34u; }
    v = __fadd_rn(c8, c35);
    if (v < b) { b = v; bp = 8u; }
    v2 = __fadd_rn(c40, c3);
    if (v2 < b2) { b2 = v2; bp2 = 40u; }
    v = __fadd_rn(c10, c33);
    if (v < b) { b = v; bp = 10u; }
    v2 = __fadd_rn(c42, c1);
    if (v2 < b2) { b2 = v2; bp2 = 42u; }
    v = __fadd_rn(c32, c11);
    if (v < b) { b = v; bp = 32u; }
    if (b2 < b) { b = b2; bp = bp2; }
    c43 = __fadd_rn(b, A[43 * 32]);
    P[43 * 32] = (uint8_t)bp;
  }
  float c44;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c8, c36);
    if (v < b) { b = v; bp = 8u; }
    v = __fadd_rn(c32, c12);
    if (v < b) { b = v; bp = 32u; }
    v = __fadd_rn(c40, c4);
    if (v < b) { b = v; bp = 40u; }
    c44 = __fadd_rn(b, A[44 * 32]);
    P[44 * 32] = (uint8_t)bp;
  }
  float c45;
  {
    float b = kTlInf, b2 = kTlInf, v, v2;
    uint32_t bp = 0xffu, bp2 = 0xffu;
    v = __fadd_rn(c4, c41);
    if (v < b) { b = v; bp = 4u; }
    v2 = __fadd_rn(c36, c9);
    if (v2 < b2) { b2 = v2; bp2 = 36u; }
    v = __fadd_rn(c8, c37);
    if (v < b) { b = v; bp = 8u; }
    v2 = __fadd_rn(c40, c5);
    if (v2 < b2) { b2 = v2; bp2 = 40u; }
    v = __fadd_rn(c12, c33);
    if (v < b) { b = v; bp = 12u; }
    v2 = __fadd_rn(c44, c1);
    if (v2 < b2) { b2 = v2; bp2 = 44u; }
    v = __fadd_rn(c32, c13);
    if (v < b) { b = v; bp = 32u; }
    if (b2 < b) { b = b2; bp = bp2; }
    c45 = __fadd_rn(b, A[45 * 32]);
    P[45 * 32] = (uint8_t)bp;
  }
  float c46;
  {
    float b = kTlInf, b2 = kTlInf, v, v2;
    uint32_t bp = 0xffu, bp2 = 0xffu;
    v = __fadd_rn(c4, c42);
    if (v < b) { b = v; bp = 4u; }
    v2 = __fadd_rn(c36, c10);
    if (v2 < b2) { b2 = v2; bp2 = 36u; }
    v = __fadd_rn(c8, c38);
    if (v < b) { b = v; bp = 8u; }
    v2 = __fadd_rn(c40, c6);
    if (v2 < b2) { b2 = v2; bp2 = 40u; }
    v = __fadd_rn(c12, c34);
    if (v < b) { b = v; bp = 12u; }
    v2 = __fadd_rn(c44, c2);
    if (v2 < b2) { b2 = v2; bp2 = 44u; }
    v = __fadd_rn(c32, c14);
    if (v < b) { b = v; bp = 32u; }
    if (b2 < b) { b = b2; bp = bp2; }
    c46 = __fadd_rn(b, A[46 * 32]);
    P[46 * 32] = (uint8_t)bp;
  }
  float c47;
  {
    float b = kTlInf, b2 = kTlInf, v, v2;
    uint32_t bp = 0xffu, bp2 = 0xffu;
    v = __fadd_rn(c2, c45);
    if (v < b) { b = v; bp = 2u; }
    v2 = __fadd_rn(c34, c13);
    if (v2 < b2) { b2 = v2; bp2 = 34u; }
    v = __fadd_rn(c4, c43);
    if (v < b) { b = v; bp = 4u; }
    v2 = __fadd_rn(c36, c11);
    if (v2 < b2) { b2 = v2; bp2 = 36u; }
    v = __fadd_rn(c6, c41);
    if (v < b) { b = v; bp = 6u; }
    v2 = __fadd_rn(c38, c9);
    if (v2 < b2) { b2 = v2; bp2 = 38u; }
    v = __fadd_rn(c8, c39);
    if (v < b) { b = v; bp = 8u; }
    v2 = __fadd_rn(c40, c7);
    if (v2 < b2) { b2 = v2; bp2 = 40u; }
    v = __fadd_rn(c10, c37);
    if (v < b) { b = v; bp = 10u; }
    v2 = __fadd_rn(c42, c5);
    if (v2 < b2) { b2 = v2; bp2 = 42u; }
    v = __fadd_rn(c12, c35);
    if (v < b) { b = v; bp = 12u; }
    v2 = __fadd_rn(c44, c3);
    if (v2 < b2) { b2 = v2; bp2 = 44u; }
    v = __fadd_rn(c14, c33);
    if (v < b) { b = v; bp = 14u; }
    v2 = __fadd_rn(c46, c1);
    if (v2 < b2) { b2 = v2; bp2 = 46u; }
    v = __fadd_rn(c32, c15);
    if (v < b) { b = v; bp = 32u; }
    if (b2 < b) { b = b2; bp = bp2; }
    c47 = __fadd_rn(b, A[47 * 32]);
    P[47 * 32] = (uint8_t)bp;
  }
  float c48;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c32, c16);
    if (v < b) { b = v; bp = 32u; }
    c48 = __fadd_rn(b, A[48 * 32]);
    P[48 * 32] = (uint8_t)bp;
  }
  float c49;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c16, c33);
    if (v < b) { b = v; bp = 16u; }
    v = __fadd_rn(c32, c17);
    if (v < b) { b = v; bp = 32u; }
    v = __fadd_rn(c48, c1);
    if (v < b) { b = v; bp = 48u; }
    c49 = __fadd_rn(b, A[49 * 32]);
    P[49 * 32] = (uint8_t)bp;
  }
  float c50;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c16, c34);
    if (v < b) { b = v; bp = 16u; }
    v = __fadd_rn(c32, c18);
    if (v < b) { b = v; bp = 32u; }
    v = __fadd_rn(c48, c2);
    if (v < b) { b = v; bp = 48u; }
    c50 = __fadd_rn(b, A[50 * 32]);
    P[50 * 32] = (uint8_t)bp;
  }
  float c51;
  {
    float b = kTlInf, b2 = kTlInf, v, v2;
    uint32_t bp = 0xffu, bp2 = 0xffu;
    v = __fadd_rn(c2, c49);
    if (v < b) { b = v; bp = 2u; }
    v2 = __fadd_rn(c34, c17);
    if (v2 < b2) { b2 = v2; bp2 = 34u; }
    v = __fadd_rn(c16, c35);
    if (v < b) { b = v; bp = 16u; }
    v2 = __fadd_rn(c48, c3);
    if (v2 < b2) { b2 = v2; bp2 = 48u; }
    v = __fadd_rn(c18, c33);
    if (v < b) { b = v; bp = 18u; }
    v2 = __fadd_rn(c50, c1);
    if (v2 < b2) { b2 = v2; bp2 = 50u; }
    v = __fadd_rn(c32, c19);
    if (v < b) { b = v; bp = 32u; }
    if (b2 < b) { b = b2; bp = bp2; }
    c51 = __fadd_rn(b, A[51 * 32]);
    P[51 * 32] = (uint8_t)bp;
  }
  float c52;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c16, c36);
    if (v < b) { b = v; bp = 16u; }
    v = __fadd_rn(c32, c20);
    if (v < b) { b = v; bp = 32u; }
    v = __fadd_rn(c48, c4);
    if (v < b) { b = v; bp = 48u; }
    c52 = __fadd_rn(b, A[52 * 32]);
    P[52 * 32] = (uint8_t)bp;
  }
  float c53;
  {
    float b = kTlInf, b2 = kTlInf, v, v2;
    uint32_t bp = 0xffu, bp2 = 0xffu;
    v = __fadd_rn(c4, c49);
    if (v < b) { b = v; bp = 4u; }
    v2 = __fadd_rn(c36, c17);
    if (v2 < b2) { b2 = v2; bp2 = 36u; }
    v = __fadd_rn(c16, c37);
    if (v < b) { b = v; bp = 16u; }
    v2 = __fadd_rn(c48, c5);
    if (v2 < b2) { b2 = v2; bp2 = 48u; }
    v = __fadd_rn(c20, c33);
    if (v < b) { b = v; bp = 20u; }
    v2 = __fadd_rn(c52, c1);
    if (v2 < b2) { b2 = v2; bp2 = 52u; }
    v = __fadd_rn(c32, c21);
    if (v < b) { b = v; bp = 32u; }
    if (b2 < b) { b = b2; bp = bp2; }
    c53 = __fadd_rn(b, A[53 * 32]);
    P[53 * 32] = (uint8_t)bp;
  }
  float c54;
  {
    float b = kTlInf, b2 = kTlInf, v, v2;
    uint32_t bp = 0xffu, bp2 = 0xffu;
    v = __fadd_rn(c4, c50);
    if (v < b) { b = v; bp = 4u; }
    v2 = __fadd_rn(c36, c18);
    if (v2 < b2) { b2 = v2; bp2 = 36u; }
    v = __fadd_rn(c16, c38);
    if (v < b) { b = v; bp = 16u; }
    v2 = __fadd_rn(c48, c6);
    if (v2 < b2) { b2 = v2; bp2 = 48u; }
    v = __fadd_rn(c20, c34);
    if (v < b) { b = v; bp = 20u; }
    v2 = __fadd_rn(c52, c2);
    if (v2 < b2) { b2 = v2; bp2 = 52u; }
    v = __fadd_rn(c32, c22);
    if (v < b) { b = v; bp = 32u; }
    if (b2 < b) { b = b2; bp = bp2; }
    c54 = __fadd_rn(b, A[54 * 32]);
    P[54 * 32] = (uint8_t)bp;
  }
  float c55;
  {
    float b = kTlInf, b2 = kTlInf, v, v2;
    uint32_t bp = 0xffu, bp2 = 0xffu;
    v = __fadd_rn(c2, c53);
    if (v < b) { b = v; bp = 2u; }
    v2 = __fadd_rn(c34, c21);
    if (v2 < b2) { b2 = v2; bp2 = 34u; }
    v = __fadd_rn(c4, c51);
    if (v < b) { b = v; bp = 4u; }
    v2 = __fadd_rn(c36, c19);
    if (v2 < b2) { b2 = v2; bp2 = 36u; }
    v = __fadd_rn(c6, c49);
    if (v < b) { b = v; bp = 6u; }
    v2 = __fadd_rn(c38, c17);
    if (v2 < b2) { b2 = v2; bp2 = 38u; }
    v = __fadd_rn(c16, c39);
    if (v < b) { b = v; bp = 16u; }
    v2 = __fadd_rn(c48, c7);
    if (v2 < b2) { b2 = v2; bp2 = 48u; }
    v = __fadd_rn(c18, c37);
    if (v < b) { b = v; bp = 18u; }
    v2 = __fadd_rn(c50, c5);
    if (v2 < b2) { b2 = v2; bp2 = 50u; }
    v = __fadd_rn(c20, c35);
    if (v < b) { b = v; bp = 20u; }
    v2 = __fadd_rn(c52, c3);
    if (v2 < b2) { b2 = v2; bp2 = 52u; }
    v = __fadd_rn(c22, c33);
    if (v < b) { b = v; bp = 22u; }
    v2 = __fadd_rn(c54, c1);
    if (v2 < b2) { b2 = v2; bp2 = 54u; }
    v = __fadd_rn(c32, c23);
    if (v < b) { b = v; bp = 32u; }
    if (b2 < b) { b = b2; bp = bp2; }
    c55 = __fadd_rn(b, A[55 * 32]);
    P[55 * 32] = (uint8_t)bp;
  }
  float c56;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c16, c40);
    if (v < b) { b = v; bp = 16u; }
    v = __fadd_rn(c32, c24);
    if (v < b) { b = v; bp = 32u; }
    v = __fadd_rn(c48, c8);
    if (v < b) { b = v; bp = 48u; }
    c56 = __fadd_rn(b, A[56 * 32]);
    P[56 * 32] = (uint8_t)bp;
  }
  float c57;
  {
    float b = kTlInf, b2 = kTlInf, v, v2;
    uint32_t bp = 0xffu, bp2 = 0xffu;
    v = __fadd_rn(c8, c49);
    if (v < b) { b = v; bp = 8u; }
    v2 = __fadd_rn(c40, c17);
    if (v2 < b2) { b2 = v2; bp2 = 40u; }
    v = __fadd_rn(c16, c41);
    if (v < b) { b = v; bp = 16u; }
    v2 = __fadd_rn(c48, c9);
    if (v2 < b2) { b2 = v2; bp2 = 48u; }
    v = __fadd_rn(c24, c33);
    if (v < b) { b = v; bp = 24u; }
    v2 = __fadd_rn(c56, c1);
    if (v2 < b2) { b2 = v2; bp2 = 56u; }
    v = __fadd_rn(c32, c25);
    if (v < b) { b = v; bp = 32u; }
    if (b2 < b) { b = b2; bp = bp2; }
    c57 = __fadd_rn(b, A[57 * 32]);
    P[57 * 32] = (uint8_t)bp;
  }
  float c58;
  {
    float b = kTlInf, b2 = kTlInf, v, v2;
    uint32_t bp = 0xffu, bp2 = 0xffu;
    v = __fadd_rn(c8, c50);
    if (v < b) { b = v; bp = 8u; }
    v2 = __fadd_rn(c40, c18);
    if (v2 < b2) { b2 = v2; bp2 = 40u; }
    v = __fadd_rn(c16, c42);
    if (v < b) { b = v; bp = 16u; }
    v2 = __fadd_rn(c48, c10);
    if (v2 < b2) { b2 = v2; bp2 = 48u; }
    v = __fadd_rn(c24, c34);
    if (v < b) { b = v; bp = 24u; }
    v2 = __fadd_rn(c56, c2);
    if (v2 < b2) { b2 = v2; bp2 = 56u; }
    v = __fadd_rn(c32, c26);
    if (v < b) { b = v; bp = 32u; }
    if (b2 < b) { b = b2; bp = bp2; }
    c58 = __fadd_rn(b, A[58 * 32]);
    P[58 * 32] = (uint8_t)bp;
  }
  float c59;
  {
    float b = kTlInf, b2 = kTlInf, v, v2;
    uint32_t bp = 0xffu, bp2 = 0xffu;
    v = __fadd_rn(c2, c57);
    if (v < b) { b = v; bp = 2u; }
    v2 = __fadd_rn(c34, c25);
    if (v2 < b2) { b2 = v2; bp2 = 34u; }
    v = __fadd_rn(c8, c51);
    if (v < b) { b = v; bp = 8u; }
    v2 = __fadd_rn(c40, c19);
    if (v2 < b2) { b2 = v2; bp2 = 40u; }
    v = __fadd_rn(c10, c49);
    if (v < b) { b = v; bp = 10u; }
    v2 = __fadd_rn(c42, c17);
    if (v2 < b2) { b2 = v2; bp2 = 42u; }
    v = __fadd_rn(c16, c43);
    if (v < b) { b = v; bp = 16u; }
    v2 = __fadd_rn(c48, c11);
    if (v2 < b2) { b2 = v2; bp2 = 48u; }
    v = __fadd_rn(c18, c41);
    if (v < b) { b = v; bp = 18u; }
    v2 = __fadd_rn(c50, c9);
    if (v2 < b2) { b2 = v2; bp2 = 50u; }
    v = __fadd_rn(c24, c35);
    if (v < b) { b = v; bp = 24u; }
    v2 = __fadd_rn(c56, c3);
    if (v2 < b2) { b2 = v2; bp2 = 56u; }
    v = __fadd_rn(c26, c33);
    if (v < b) { b = v; bp = 26u; }
    v2 = __fadd_rn(c58, c1);
    if (v2 < b2) { b2 = v2; bp2 = 58u; }
    v = __fadd_rn(c32, c27);
    if (v < b) { b = v; bp = 32u; }
    if (b2 < b) { b = b2; bp = bp2; }
    c59 = __fadd_rn(b, A[59 * 32]);
    P[59 * 32] = (uint8_t)bp;
  }
  float c60;
  {
    float b = kTlInf, b2 = kTlInf, v, v2;
    uint32_t bp = 0xffu, bp2 = 0xffu;
    v = __fadd_rn(c8, c52);
    if (v < b) { b = v; bp = 8u; }
    v2 = __fadd_rn(c40, c20);
    if (v2 < b2) { b2 = v2; bp2 = 40u; }
    v = __fadd_rn(c16, c44);
    if (v < b) { b = v; bp = 16u; }
    v2 = __fadd_rn(c48, c12);
    if (v2 < b2) { b2 = v2; bp2 = 48u; }
    v = __fadd_rn(c24, c36);
    if (v < b) { b = v; bp = 24u; }
    v2 = __fadd_rn(c56, c4);
    if (v2 < b2) { b2 = v2; bp2 = 56u; }
    v = __fadd_rn(c32, c28);
    if (v < b) { b = v; bp = 32u; }
    if (b2 < b) { b = b2; bp = bp2; }
    c60 = __fadd_rn(b, A[60 * 32]);
    P[60 * 32] = (uint8_t)bp;
  }
  float c61;
  {
    float b = kTlInf, b2 = kTlInf, v, v2;
    uint32_t bp = 0xffu, bp2 = 0xffu;
    v = __fadd_rn(c4, c57);
    if (v < b) { b = v; bp = 4u; }
    v2 = __fadd_rn(c36, c25);
    if (v2 < b2) { b2 = v2; bp2 = 36u; }
    v = __fadd_rn(c8, c53);
    if (v < b) { b = v; bp = 8u; }
    v2 = __fadd_rn(c40, c21);
    if (v2 < b2) { b2 = v2; bp2 = 40u; }
    v = __fadd_rn(c12, c49);
    if (v < b) { b = v; bp = 12u; }
    v2 = __fadd_rn(c44, c17);
    if (v2 < b2) { b2 = v2; bp2 = 44u; }
    v = __fadd_rn(c16, c45);
    if (v < b) { b = v; bp = 16u; }
    v2 = __fadd_rn(c48, c13);
    if (v2 < b2) { b2 = v2; bp2 = 48u; }
    v = __fadd_rn(c20, c41);
    if (v < b) { b = v; bp = 20u; }
    v2 = __fadd_rn(c52, c9);
    if (v2 < b2) { b2 = v2; bp2 = 52u; }
    v = __fadd_rn(c24, c37);
    if (v < b) { b = v; bp = 24u; }
    v2 = __fadd_rn(c56, c5);
    if (v2 < b2) { b2 = v2; bp2 = 56u; }
    v = __fadd_rn(c28, c33);
    if (v < b) { b = v; bp = 28u; }
    v2 = __fadd_rn(c60, c1);
    if (v2 < b2) { b2 = v2; bp2 = 60u; }
    v = __fadd_rn(c32, c29);
    if (v < b) { b = v; bp = 32u; }
    if (b2 < b) { b = b2; bp = bp2; }
    c61 = __fadd_rn(b, A[61 * 32]);
    P[61 * 32] = (uint8_t)bp;
  }
  float c62;
  {
    float b = kTlInf, b2 = kTlInf, v, v2;
    uint32_t bp = 0xffu, bp2 = 0xffu;
    v = __fadd_rn(c4, c58);
    if (v < b) { b = v; bp = 4u; }
    v2 = __fadd_rn(c36, c26);
    if (v2 < b2) { b2 = v2; bp2 = 36u; }
    v = __fadd_rn(c8, c54);
    if (v < b) { b = v; bp = 8u; }
    v2 = __fadd_rn(c40, c22);
    if (v2 < b2) { b2 = v2; bp2 = 40u; }
    v = __fadd_rn(c12, c50);
    if (v < b) { b = v; bp = 12u; }
    v2 = __fadd_rn(c44, c18);
    if (v2 < b2) { b2 = v2; bp2 = 44u; }
    v = __fadd_rn(c16, c46);
    if (v < b) { b = v; bp = 16u; }
    v2 = __fadd_rn(c48, c14);
    if (v2 < b2) { b2 = v2; bp2 = 48u; }
    v = __fadd_rn(c20, c42);
    if (v < b) { b = v; bp = 20u; }
    v2 = __fadd_rn(c52, c10);
    if (v2 < b2) { b2 = v2; bp2 = 52u; }
    v = __fadd_rn(c24, c38);
    if (v < b) { b = v; bp = 24u; }
    v2 = __fadd_rn(c56, c6);
    if (v2 < b2) { b2 = v2; bp2 = 56u; }
    v = __fadd_rn(c28, c34);
    if (v < b) { b = v; bp = 28u; }
    v2 = __fadd_rn(c60, c2);
    if (v2 < b2) { b2 = v2; bp2 = 60u; }
    v = __fadd_rn(c32, c30);
    if (v < b) { b = v; bp = 32u; }
    if (b2 < b) { b = b2; bp = bp2; }
    c62 = __fadd_rn(b, A[62 * 32]);
    P[62 * 32] = (uint8_t)bp;
  }
  {
    float b = kTlInf, b2 = kTlInf, v, v2;
    uint32_t bp = 0xffu, bp2 = 0xffu;
    v = __fadd_rn(c2, c61);
    if (v < b) { b = v; bp = 2u; }
    v2 = __fadd_rn(c34, c29);
    if (v2 < b2) { b2 = v2; bp2 = 34u; }
    v = __fadd_rn(c4, c59);
    if (v < b) { b = v; bp = 4u; }
    v2 = __fadd_rn(c36, c27);
    if (v2 < b2) { b2 = v2; bp2 = 36u; }
    v = __fadd_rn(c6, c57);
    if (v < b) { b = v; bp = 6u; }
    v2 = __fadd_rn(c38, c25);
    if (v2 < b2) { b2 = v2; bp2 = 38u; }
    v = __fadd_rn(c8, c55);
    if (v < b) { b = v; bp = 8u; }
    v2 = __fadd_rn(c40, c23);
    if (v2 < b2) { b2 = v2; bp2 = 40u; }
    v = __fadd_rn(c10, c53);
    if (v < b) { b = v; bp = 10u; }
    v2 = __fadd_rn(c42, c21);
    if (v2 < b2) { b2 = v2; bp2 = 42u; }
    v = __fadd_rn(c12, c51);
    if (v < b) { b = v; bp = 12u; }
    v2 = __fadd_rn(c44, c19);
    if (v2 < b2) { b2 = v2; bp2 = 44u; }
    v = __fadd_rn(c14, c49);
    if (v < b) { b = v; bp = 14u; }
    v2 = __fadd_rn(c46, c17);
    if (v2 < b2) { b2 = v2; bp2 = 46u; }
    v = __fadd_rn(c16, c47);
    if (v < b) { b = v; bp = 16u; }
    v2 = __fadd_rn(c48, c15);
    if (v2 < b2) { b2 = v2; bp2 = 48u; }
    v = __fadd_rn(c18, c45);
    if (v < b) { b = v; bp = 18u; }
    v2 = __fadd_rn(c50, c13);
    if (v2 < b2) { b2 = v2; bp2 = 50u; }
    v = __fadd_rn(c20, c43);
    if (v < b) { b = v; bp = 20u; }
    v2 = __fadd_rn(c52, c11);
    if (v2 < b2) { b2 = v2; bp2 = 52u; }
    v = __fadd_rn(c22, c41);
    if (v < b) { b = v; bp = 22u; }
    v2 = __fadd_rn(c54, c9);
    if (v2 < b2) { b2 = v2; bp2 = 54u; }
    v = __fadd_rn(c24, c39);
    if (v < b) { b = v; bp = 24u; }
    v2 = __fadd_rn(c56, c7);
    if (v2 < b2) { b2 = v2; bp2 = 56u; }
    v = __fadd_rn(c26, c37);
    if (v < b) { b = v; bp = 26u; }
    v2 = __fadd_rn(c58, c5);
    if (v2 < b2) { b2 = v2; bp2 = 58u; }
    v = __fadd_rn(c28, c35);
    if (v < b) { b = v; bp = 28u; }
    v2 = __fadd_rn(c60, c3);
    if (v2 < b2) { b2 = v2; bp2 = 60u; }
    v = __fadd_rn(c30, c33);
    if (v < b) { b = v; bp = 30u; }
    v2 = __fadd_rn(c62, c1);
    if (v2 < b2) { b2 = v2; bp2 = 62u; }
    v = __fadd_rn(c32, c31);
    if (v < b) { b = v; bp = 32u; }
    if (b2 < b) { b = b2; bp = bp2; }
    P[63 * 32] = (uint8_t)bp;
  }
}

// 7 leaves: 966 split evaluations.
__device__ __forceinline__ void dp_unrolled_7(const float* __restrict__ A, uint8_t* __restrict__ P) {
  const float c1 = 0.0f;
  const float c2 = 0.0f;
  float c3;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c2, c1);
    if (v < b) { b = v; bp = 2u; }
    c3 = __fadd_rn(b, A[3 * 32]);
    P[3 * 32] = (uint8_t)bp;
  }
  const float c4 = 0.0f;
  float c5;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c4, c1);
    if (v < b) { b = v; bp = 4u; }
    c5 = __fadd_rn(b, A[5 * 32]);
    P[5 * 32] = (uint8_t)bp;
  }
  float c6;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c4, c2);
    if (v < b) { b = v; bp = 4u; }
    c6 = __fadd_rn(b, A[6 * 32]);
    P[6 * 32] = (uint8_t)bp;
  }
  float c7;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c2, c5);
    if (v < b) { b = v; bp = 2u; }
    v = __fadd_rn(c4, c3);
    if (v < b) { b = v; bp = 4u; }
    v = __fadd_rn(c6, c1);
    if (v < b) { b = v; bp = 6u; }
    c7 = __fadd_rn(b, A[7 * 32]);
    P[7 * 32] = (uint8_t)bp;
  }
  const float c8 = 0.0f;
  float c9;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c8, c1);
    if (v < b) { b = v; bp = 8u; }
    c9 = __fadd_rn(b, A[9 * 32]);
    P[9 * 32] = (uint8_t)bp;
  }
  float c10;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c8, c2);
    if (v < b) { b = v; bp = 8u; }
    c10 = __fadd_rn(b, A[10 * 32]);
    P[10 * 32] = (uint8_t)bp;
  }
  float c11;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c2, c9);
    if (v < b) { b = v; bp = 2u; }
    v = __fadd_rn(c8, c3);
    if (v < b) { b = v; bp = 8u; }
    v = __fadd_rn(c10, c1);
    if (v < b) { b = v; bp = 10u; }
    c11 = __fadd_rn(b, A[11 * 32]);
    P[11 * 32] = (uint8_t)bp;
  }
  float c12;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c8, c4);
    if (v < b) { b = v; bp = 8u; }
    c12 = __fadd_rn(b, A[12 * 32]);
    P[12 * 32] = (uint8_t)bp;
  }
  float c13;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c4, c9);
    if (v < b) { b = v; bp = 4u; }
    v = __fadd_rn(c8, c5);
    if (v < b) { b = v; bp = 8u; }
    v = __fadd_rn(c12, c1);
    if (v < b) { b = v; bp = 12u; }
    c13 = __fadd_rn(b, A[13 * 32]);
    P[13 * 32] = (uint8_t)bp;
  }
  float c14;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c4, c10);
    if (v < b) { b = v; bp = 4u; }
    v = __fadd_rn(c8, c6);
    if (v < b) { b = v; bp = 8u; }
    v = __fadd_rn(c12, c2);
    if (v < b) { b = v; bp = 12u; }
    c14 = __fadd_rn(b, A[14 * 32]);
    P[14 * 32] = (uint8_t)bp;
  }
  float c15;
  {
    float b = kTlInf, b2 = kTlInf, v, v2;
    uint32_t bp = 0xffu, bp2 = 0xffu;
    v = __fadd_rn(c2, c13);
    if (v < b) { b = v; bp = 2u; }
    v2 = __fadd_rn(c10, c5);
    if (v2 < b2) { b2 = v2; bp2 = 10u; }
    v = __fadd_rn(c4, c11);
    if (v < b) { b = v; bp = 4u; }
    v2 = __fadd_rn(c12, c3);
    if (v2 < b2) { b2 = v2; bp2 = 12u; }
    v = __fadd_rn(c6, c9);
    if (v < b) { b = v; bp = 6u; }
    v2 = __fadd_rn(c14, c1);
    if (v2 < b2) { b2 = v2; bp2 = 14u; }
    v = __fadd_rn(c8, c7);
    if (v < b) { b = v; bp = 8u; }
    if (b2 < b) { b = b2; bp = bp2; }
    c15 = __fadd_rn(b, A[15 * 32]);
    P[15 * 32] = (uint8_t)bp;
  }
  const float c16 = 0.0f;
  float c17;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c16, c1);
    if (v < b) { b = v; bp = 16u; }
    c17 = __fadd_rn(b, A[17 * 32]);
    P[17 * 32] = (uint8_t)bp;
  }
  float c18;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c16, c2);
    if (v < b) { b = v; bp = 16u; }
    c18 = __fadd_rn(b, A[18 * 32]);
    P[18 * 32] = (uint8_t)bp;
  }
  float c19;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c2, c17);
    if (v < b) { b = v; bp = 2u; }
    v = __fadd_rn(c16, c3);
    if (v < b) { b = v; bp = 16u; }
    v = __fadd_rn(c18, c1);
    if (v < b) { b = v; bp = 18u; }
    c19 = __fadd_rn(b, A[19 * 32]);
    P[19 * 32] = (uint8_t)bp;
  }
  float c20;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c16, c4);
    if (v < b) { b = v; bp = 16u; }
    c20 = __fadd_rn(b, A[20 * 32]);
    P[20 * 32] = (uint8_t)bp;
  }
  float c21;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c4, c17);
    if (v < b) { b = v; bp = 4u; }
    v = __fadd_rn(c16, c5);
    if (v < b) { b = v; bp = 16u; }
    v = __fadd_rn(c20, c1);
    if (v < b) { b = v; bp = 20u; }
    c21 = __fadd_rn(b, A[21 * 32]);
    P[21 * 32] = (uint8_t)bp;
  }
  float c22;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c4, c18);
    if (v < b) { b = v; bp = 4u; }
    v = __fadd_rn(c16, c6);
    if (v < b) { b = v; bp = 16u; }
    v = __fadd_rn(c20, c2);
    if (v < b) { b = v; bp = 20u; }
    c22 = __fadd_rn(b, A[22 * 32]);
    P[22 * 32] = (uint8_t)bp;
  }
  float c23;
  {
    float b = kTlInf, b2 = kTlInf, v, v2;
    uint32_t bp = 0xffu, bp2 = 0xffu;
    v = __fadd_rn(c2, c21);
    if (v < b) { b = v; bp = 2u; }
    v2 = __fadd_rn(c18, c5);
    if (v2 < b2) { b2 = v2; bp2 = 18u; }
    v = __fadd_rn(c4, c19);
    if (v < b) { b = v; bp = 4u; }
    v2 = __fadd_rn(c20, c3);
    if (v2 < b2) { b2 = v2; bp2 = 20u; }
    v = __fadd_rn(c6, c17);
    if (v < b) { b = v; bp = 6u; }
    v2 = __fadd_rn(c22, c1);
    if (v2 < b2) { b2 = v2; bp2 = 22u; }
    v = __fadd_rn(c16, c7);
    if (v < b) { b = v; bp = 16u; }
    if (b2 < b) { b = b2; bp = bp2; }
    c23 = __fadd_rn(b, A[23 * 32]);
    P[23 * 32] = (uint8_t)bp;
  }
  float c24;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c16, c8);
    if (v < b) { b = v; bp = 16u; }
    c24 = __fadd_rn(b, A[24 * 32]);
    P[24 * 32] = (uint8_t)bp;
  }
  float c25;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c8, c17);
    if (v < b) { b = v; bp = 8u; }
    v = __fadd_rn(c16, c9);
    if (v < b) { b = v; bp = 16u; }
    v = __fadd_rn(c24, c1);
    if (v < b) { b = v; bp = 24u; }
    c25 = __fadd_rn(b, A[25 * 32]);
    P[25 * 32] = (uint8_t)bp;
  }
  float c26;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c8, c18);
    if (v < b) { b = v; bp = 8u; }
    v = __fadd_rn(c16, c10);
    if (v < b) { b = v; bp = 16u; }
    v = __fadd_rn(c24, c2);
    if (v < b) { b = v; bp = 24u; }
    c26 = __fadd_rn(b, A[26 * 32]);
    P[26 * 32] = (uint8_t)bp;
  }
  float c27;
  {
    float b = kTlInf, b2 = kTlInf, v, v2;
    uint32_t bp = 0xffu, bp2 = 0xffu;
    v = __fadd_rn(c2, c25);
    if (v < b) { b = v; bp = 2u; }
    v2 = __fadd_rn(c18, c9);
    if (v2 < b2) { b2 = v2; bp2 = 18u; }
    v = __fadd_rn(c8, c19);
    if (v < b) { b = v; bp = 8u; }
    v2 = __fadd_rn(c24, c3);
    if (v2 < b2) { b2 = v2; bp2 = 24u; }
    v = __fadd_rn(c10, c17);
    if (v < b) { b = v; bp = 10u; }
    v2 = __fadd_rn(c26, c1);
    if (v2 < b2) { b2 = v2; bp2 = 26u; }
    v = __fadd_rn(c16, c11);
    if (v < b) { b = v; bp = 16u; }
    if (b2 < b) { b = b2; bp = bp2; }
    c27 = __fadd_rn(b, A[27 * 32]);
    P[27 * 32] = (uint8_t)bp;
  }
  float c28;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c8, c20);
    if (v < b) { b = v; bp = 8u; }
    v = __fadd_rn(c16, c12);
    if (v < b) { b = v; bp = 16u; }
    v = __fadd_rn(c24, c4);
    if (v < b) { b = v; bp = 24u; }
    c28 = __fadd_rn(b, A[28 * 32]);
    P[28 * 32] = (uint8_t)bp;
  }
  float c29;
  {
    float b = kTlInf, b2 = kTlInf, v, v2;
    uint32_t bp = 0xffu, bp2 = 0xffu;
    v = __fadd_rn(c4, c25);
    if (v < b) { b = v; bp = 4u; }
    v2 = __fadd_rn(c20, c9);
    if (v2 < b2) { b2 = v2; bp2 = 20u; }
    v = __fadd_rn(c8, c21);
    if (v < b) { b = v; bp = 8u; }
    v2 = __fadd_rn(c24, c5);
    if (v2 < b2) { b2 = v2; bp2 = 24u; }
    v = __fadd_rn(c12, c17);
    if (v < b) { b = v; bp = 12u; }
    v2 = __fadd_rn(c28, c1);
    if (v2 < b2) { b2 = v2; bp2 = 28u; }
    v = __fadd_rn(c16, c13);
    if (v < b) { b = v; bp = 16u; }
    if (b2 < b) { b = b2; bp = bp2; }
    c29 = __fadd_rn(b, A[29 * 32]);
    P[29 * 32] = (uint8_t)bp;
  }
  float c30;
  {
    float b = kTlInf, b2 = kTlInf, v, v2;
    uint32_t bp = 0xffu, bp2 = 0xffu;
    v = __fadd_rn(c4, c26);
    if (v < b) { b = v; bp = 4u; }
    v2 = __fadd_rn(c20, c10);
    if (v2 < b2) { b2 = v2; bp2 = 20u; }
    v = __fadd_rn(c8, c22);
    if (v < b) { b = v; bp = 8u; }
    v2 = __fadd_rn(c24, c6);
    if (v2 < b2) { b2 = v2; bp2 = 24u; }
    v = __fadd_rn(c12, c18);
    if (v < b) { b = v; bp = 12u; }
    v2 = __fadd_rn(c28, c2);
    if (v2 < b2) { b2 = v2; bp2 = 28u; }
    v = __fadd_rn(c16, c14);
    if (v < b) { b = v; bp = 16u; }
    if (b2 < b) { b = b2; bp = bp2; }
    c30 = __fadd_rn(b, A[30 * 32]);
    P[30 * 32] = (uint8_t)bp;
  }
  float c31;
  {
    float b = kTlInf, b2 = kTlInf, v, v2;
    uint32_t bp = 0xffu, bp2 = 0xffu;
    v = __fadd_rn(c2, c29);
    if (v < b) { b = v; bp = 2u; }
    v2 = __fadd_rn(c18, c13);
    if (v2 < b2) { b2 = v2; bp2 = 18u; }
    v = __fadd_rn(c4, c27);
    if (v < b) { b = v; bp = 4u; }
    v2 = __fadd_rn(c20, c11);
    if (v2 < b2) { b2 = v2; bp2 = 20u; }
    v = __fadd_rn(c6, c25);
    if (v < b) { b = v; bp = 6u; }
    v2 = __fadd_rn(c22, c9);
    if (v2 < b2) { b2 = v2; bp2 = 22u; }
    v = __fadd_rn(c8, c23);
    if (v < b) { b = v; bp = 8u; }
    v2 = __fadd_rn(c24, c7);
    if (v2 < b2) { b2 = v2; bp2 = 24u; }
    v = __fadd_rn(c10, c21);
    if (v < b) { b = v; bp = 10u; }
    v2 = __fadd_rn(c26, c5);
    if (v2 < b2) { b2 = v2; bp2 = 26u; }
    v = __fadd_rn(c12, c19);
    if (v < b) { b = v; bp = 12u; }
    v2 = __fadd_rn(c28, c3);
    if (v2 < b2) { b2 = v2; bp2 = 28u; }
    v = __fadd_rn(c14, c17);
    if (v < b) { b = v; bp = 14u; }
    v2 = __fadd_rn(c30, c1);
    if (v2 < b2) { b2 = v2; bp2 = 30u; }
    v = __fadd_rn(c16, c15);
    if (v < b) { b = v; bp = 16u; }
    if (b2 < b) { b = b2; bp = bp2; }
    c31 = __fadd_rn(b, A[31 * 32]);
    P[31 * 32] = (uint8_t)bp;
  }
  const float c32 = 0.0f;
  float c33;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c32, c1);
    if (v < b) { b = v; bp = 32u; }
    c33 = __fadd_rn(b, A[33 * 32]);
    P[33 * 32] = (uint8_t)bp;
  }
  float c34;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c32, c2);
    if (v < b) { b = v; bp = 32u; }
    c34 = __fadd_rn(b, A[34 * 32]);
    P[34 * 32] = (uint8_t)bp;
  }
  float c35;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c2, c33);
    if (v < b) { b = v; bp = 2u; }
    v = __fadd_rn(c32, c3);
    if (v < b) { b = v; bp = 32u; }
    v = __fadd_rn(c34, c1);
    if (v < b) { b = v; bp = 34u; }
    c35 = __fadd_rn(b, A[35 * 32]);
    P[35 * 32] = (uint8_t)bp;
  }
  float c36;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c32, c4);
    if (v < b) { b = v; bp = 32u; }
    c36 = __fadd_rn(b, A[36 * 32]);
    P[36 * 32] = (uint8_t)bp;
  }
  float c37;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c4, c33);
    if (v < b) { b = v; bp = 4u; }
    v = __fadd_rn(c32, c5);
    if (v < b) { b = v; bp = 32u; }
    v = __fadd_rn(c36, c1);
    if (v < b) { b = v; bp = 36u; }
    c37 = __fadd_rn(b, A[37 * 32]);
    P[37 * 32] = (uint8_t)bp;
  }
  float c38;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c4, c34);
    if (v < b) { b = v; bp = 4u; }
    v = __fadd_rn(c32, c6);
    if (v < b) { b = v; bp = 32u; }
    v = __fadd_rn(c36, c2);
    if (v < b) { b = v; bp = 36u; }
    c38 = __fadd_rn(b, A[38 * 32]);
    P[38 * 32] = (uint8_t)bp;
  }
  float c39;
  {
    float b = kTlInf, b2 = kTlInf, v, v2;
    uint32_t bp = 0xffu, bp2 = 0xffu;
    v = __fadd_rn(c2, c37);
    if (v < b) { b = v; bp = 2u; }
    v2 = __fadd_rn(c34, c5);
    if (v2 < b2) { b2 = v2; bp2 = 34u; }
    v = __fadd_rn(c4, c35);
    if (v < b) { b = v; bp = 4u; }
    v2 = __fadd_rn(c36, c3);
    if (v2 < b2) { b2 = v2; bp2 = 36u; }
    v = __fadd_rn(c6, c33);
    if (v < b) { b = v; bp = 6u; }
    v2 = __fadd_rn(c38, c1);
    if (v2 < b2) { b2 = v2; bp2 = 38u; }
    v = __fadd_rn(c32, c7);
    if (v < b) { b = v; bp = 32u; }
    if (b2 < b) { b = b2; bp = bp2; }
    c39 = __fadd_rn(b, A[39 * 32]);
    P[39 * 32] = (uint8_t)bp;
  }
  float c40;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c32, c8);
    if (v < b) { b = v; bp = 32u; }
    c40 = __fadd_rn(b, A[40 * 32]);
    P[40 * 32] = (uint8_t)bp;
  }
  float c41;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c8, c33);
    if (v < b) { b = v; bp = 8u; }
    v = __fadd_rn(c32, c9);
    if (v < b) { b = v; bp = 32u; }
    v = __fadd_rn(c40, c1);
    if (v < b) { b = v; bp = 40u; }
    c41 = __fadd_rn(b, A[41 * 32]);
    P[41 * 32] = (uint8_t)bp;
  }
  float c42;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c8, c34);
    if (v < b) { b = v; bp = 8u; }
    v = __fadd_rn(c32, c10);
    if (v < b) { b = v; bp = 32u; }
    v = __fadd_rn(c40, c2);
    if (v < b) { b = v; bp = 40u; }
    c42 = __fadd_rn(b, A[42 * 32]);
    P[42 * 32] = (uint8_t)bp;
  }
  float c43;
  {
    float b = kTlInf, b2 = kTlInf, v, v2;
    uint32_t bp = 0xffu, bp2 = 0xffu;
    v = __fadd_rn(c2, c41);
    if (v < b) { b = v; bp = 2u; }
    v2 = __fadd_rn(c34, c9);
    if (v2 < b2) { b2 = v2; bp2 = 34u; }
    v = __fadd_rn(c8, c35);
    if (v < b) { b = v; bp = 8u; }
    v2 = __fadd_rn(c40, c3);
    if (v2 < b2) { b2 = v2; bp2 = 40u; }
    v = __fadd_rn(c10, c33);
    if (v < b) { b = v; bp = 10u; }
    v2 = __fadd_rn(c42, c1);
    if (v2 < b2) { b2 = v2; bp2 = 42u; }
    v = __fadd_rn(c32, c11);
    if (v < b) { b = v; bp = 32u; }
    if (b2 < b) { b = b2; bp = bp2; }
    c43 = __fadd_rn(b, A[43 * 32]);
    P[43 * 32] = (uint8_t)bp;
  }
  float c44;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c8, c36);
    if (v < b) { b = v; bp = 8u; }
    v = __fadd_rn(c32, c12);
    if (v < b) { b = v; bp = 32u; }
    v = __fadd_rn(c40, c4);
    if (v < b) { b = v; bp = 40u; }
    c44 = __fadd_rn(b, A[44 * 32]);
    P[44 * 32] = (uint8_t)bp;
  }
  float c45;
  {
    float b = kTlInf, b2 = kTlInf, v, v2;
    uint32_t bp = 0xffu, bp2 = 0xffu;
    v = __fadd_rn(c4, c41);
    if (v < b) { b = v; bp = 4u; }
    v2 = __fadd_rn(c36, c9);
    if (v2 < b2) { b2 = v2; bp2 = 36u; }
    v = __fadd_rn(c8, c37);
    if (v < b) { b = v; bp = 8u; }
    v2 = __fadd_rn(c40, c5);
    if (v2 < b2) { b2 = v2; bp2 = 40u; }
    v = __fadd_rn(c12, c33);
    if (v < b) { b = v; bp = 12u; }
    v2 = __fadd_rn(c44, c1);
    if (v2 < b2) { b2 = v2; bp2 = 44u; }
    v = __fadd_rn(c32, c13);
    if (v < b) { b = v; bp = 32u; }
    if (b2 < b) { b = b2; bp = bp2; }
    c45 = __fadd_rn(b, A[45 * 32]);
    P[45 * 32] = (uint8_t)bp;
  }
  float c46;
  {
    float b = kTlInf, b2 = kTlInf, v, v2;
    uint32_t bp = 0xffu, bp2 = 0xffu;
    v = __fadd_rn(c4, c42);
    if (v < b) { b = v; bp = 4u; }
    v2 = __fadd_rn(c36, c10);
    if (v2 < b2) { b2 = v2; bp2 = 36u; }
    v = __fadd_rn(c8, c38);
    if (v < b) { b = v; bp = 8u; }
    v2 = __fadd_rn(c40, c6);
    if (v2 < b2) { b2 = v2; bp2 = 40u; }
    v = __fadd_rn(c12, c34);
    if (v < b) { b = v; bp = 12u; }
    v2 = __fadd_rn(c44, c2);
    if (v2 < b2) { b2 = v2; bp2 = 44u; }
    v = __fadd_rn(c32, c14);
    if (v < b) { b = v; bp = 32u; }
    if (b2 < b) { b = b2; bp = bp2; }
    c46 = __fadd_rn(b, A[46 * 32]);
    P[46 * 32] = (uint8_t)bp;
  }
  float c47;
  {
    float b = kTlInf, b2 = kTlInf, v, v2;
    uint32_t bp = 0xffu, bp2 = 0xffu;
    v = __fadd_rn(c2, c45);
    if (v < b) { b = v; bp = 2u; }
    v2 = __fadd_rn(c34, c13);
    if (v2 < b2) { b2 = v2; bp2 = 34u; }
    v = __fadd_rn(c4, c43);
    if (v < b) { b = v; bp = 4u; }
    v2 = __fadd_rn(c36, c11);
    if (v2 < b2) { b2 = v2; bp2 = 36u; }
    v = __fadd_rn(c6, c41);
    if (v < b) { b = v; bp = 6u; }
    v2 = __fadd_rn(c38, c9);
    if (v2 < b2) { b2 = v2; bp2 = 38u; }
    v = __fadd_rn(c8, c39);
    if (v < b) { b = v; bp = 8u; }
    v2 = __fadd_rn(c40, c7);
    if (v2 < b2) { b2 = v2; bp2 = 40u; }
    v = __fadd_rn(c10, c37);
    if (v < b) { b = v; bp = 10u; }
    v2 = __fadd_rn(c42, c5);
    if (v2 < b2) { b2 = v2; bp2 = 42u; }
    v = __fadd_rn(c12, c35);
    if (v < b) { b = v; bp = 12u; }
    v2 = __fadd_rn(c44, c3);
    if (v2 < b2) { b2 = v2; bp2 = 44u; }
    v = __fadd_rn(c14, c33);
    if (v < b) { b = v; bp = 14u; }
    v2 = __fadd_rn(c46, c1);
    if (v2 < b2) { b2 = v2; bp2 = 46u; }
    v = __fadd_rn(c32, c15);
    if (v < b) { b = v; bp = 32u; }
    if (b2 < b) { b = b2; bp = bp2; }
    c47 = __fadd_rn(b, A[47 * 32]);
    P[47 * 32] = (uint8_t)bp;
  }
  float c48;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c32, c16);
    if (v < b) { b = v; bp = 32u; }
    c48 = __fadd_rn(b, A[48 * 32]);
    P[48 * 32] = (uint8_t)bp;
  }
  float c49;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c16, c33);
    if (v < b) { b = v; bp = 16u; }
    v = __fadd_rn(c32, c17);
    if (v < b) { b = v; bp = 32u; }
    v = __fadd_rn(c48, c1);
    if (v < b) { b = v; bp = 48u; }
    c49 = __fadd_rn(b, A[49 * 32]);
    P[49 * 32] = (uint8_t)bp;
  }
  float c50;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c16, c34);
    if (v < b) { b = v; bp = 16u; }
    v = __fadd_rn(c32, c18);
    if (v < b) { b = v; bp = 32u; }
    v = __fadd_rn(c48, c2);
    if (v < b) { b = v; bp = 48u; }
    c50 = __fadd_rn(b, A[50 * 32]);
    P[50 * 32] = (uint8_t)bp;
  }
  float c51;
  {
    float b = kTlInf, b2 = kTlInf, v, v2;
    uint32_t bp = 0xffu, bp2 = 0xffu;
    v = __fadd_rn(c2, c49);
    if (v < b) { b = v; bp = 2u; }
    v2 = __fadd_rn(c34, c17);
    if (v2 < b2) { b2 = v2; bp2 = 34u; }
    v = __fadd_rn(c16, c35);
    if (v < b) { b = v; bp = 16u; }
    v2 = __fadd_rn(c48, c3);
    if (v2 < b2) { b2 = v2; bp2 = 48u; }
    v = __fadd_rn(c18, c33);
    if (v < b) { b = v; bp = 18u; }
    v2 = __fadd_rn(c50, c1);
    if (v2 < b2) { b2 = v2; bp2 = 50u; }
    v = __fadd_rn(c32, c19);
    if (v < b) { b = v; bp = 32u; }
    if (b2 < b) { b = b2; bp = bp2; }
    c51 = __fadd_rn(b, A[51 * 32]);
    P[51 * 32] = (uint8_t)bp;
  }
  float c52;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c16, c36);
    if (v < b) { b = v; bp = 16u; }
    v = __fadd_rn(c32, c20);
    if (v < b) { b = v; bp = 32u; }
    v = __fadd_rn(c48, c4);
    if (v < b) { b = v; bp = 48u; }
    c52 = __fadd_rn(b, A[52 * 32]);
    P[52 * 32] = (uint8_t)bp;
  }
  float c53;
  {
    float b = kTlInf, b2 = kTlInf, v, v2;
    uint32_t bp = 0xffu, bp2 = 0xffu;
    v = __fadd_rn(c4, c49);
    if (v < b) { b = v; bp = 4u; }
    v2 = __fadd_rn(c36, c17);
    if (v2 < b2) { b2 = v2; bp2 = 36u; }
    v = __fadd_rn(c16, c37);
    if (v < b) { b = v; bp = 16u; }
    v2 = __fadd_rn(c48, c5);
    if (v2 < b2) { b2 = v2; bp2 = 48u; }
    v = __fadd_rn(c20, c33);
    if (v < b) { b = v; bp = 20u; }
    v2 = __fadd_rn(c52, c1);
    if (v2 < b2) { b2 = v2; bp2 = 52u; }
    v = __fadd_rn(c32, c21);
    if (v < b) { b = v; bp = 32u; }
    if (b2 < b) { b = b2; bp = bp2; }
    c53 = __fadd_rn(b, A[53 * 32]);
    P[53 * 32] = (uint8_t)bp;
  }
  float c54;
  {
    float b = kTlInf, b2 = kTlInf, v, v2;
    uint32_t bp = 0xffu, bp2 = 0xffu;
    v = __fadd_rn(c4, c50);
    if (v < b) { b = v; bp = 4u; }
    v2 = __fadd_rn(c36, c18);
    if (v2 < b2) { b2 = v2; bp2 = 36u; }
    v = __fadd_rn(c16, c38);
    if (v < b) { b = v; bp = 16u; }
    v2 = __fadd_rn(c48, c6);
    if (v2 < b2) { b2 = v2; bp2 = 48u; }
    v = __fadd_rn(c20, c34);
    if (v < b) { b = v; bp = 20u; }
    v2 = __fadd_rn(c52, c2);
    if (v2 < b2) { b2 = v2; bp2 = 52u; }
    v = __fadd_rn(c32, c22);
    if (v < b) { b = v; bp = 32u; }
    if (b2 < b) { b = b2; bp = bp2; }
    c54 = __fadd_rn(b, A[54 * 32]);
    P[54 * 32] = (uint8_t)bp;
  }
  float c55;
  {
    float b = kTlInf, b2 = kTlInf, v, v2;
    uint32_t bp = 0xffu, bp2 = 0xffu;
    v = __fadd_rn(c2, c53);
    if (v < b) { b = v; bp = 2u; }
    v2 = __fadd_rn(c34, c21);
    if (v2 < b2) { b2 = v2; bp2 = 34u; }
    v = __fadd_rn(c4, c51);
    if (v < b) { b = v; bp = 4u; }
    v2 = __fadd_rn(c36, c19);
    if (v2 < b2) { b2 = v2; bp2 = 36u; }
    v = __fadd_rn(c6, c49);
    if (v < b) { b = v; bp = 6u; }
    v2 = __fadd_rn(c38, c17);
    if (v2 < b2) { b2 = v2; bp2 = 38u; }
    v = __fadd_rn(c16, c39);
    if (v < b) { b = v; bp = 16u; }
    v2 = __fadd_rn(c48, c7);
    if (v2 < b2) { b2 = v2; bp2 = 48u; }
    v = __fadd_rn(c18, c37);
    if (v < b) { b = v; bp = 18u; }
    v2 = __fadd_rn(c50, c5);
    if (v2 < b2) { b2 = v2; bp2 = 50u; }
    v = __fadd_rn(c20, c35);
    if (v < b) { b = v; bp = 20u; }
    v2 = __fadd_rn(c52, c3);
    if (v2 < b2) { b2 = v2; bp2 = 52u; }
    v = __fadd_rn(c22, c33);
    if (v < b) { b = v; bp = 22u; }
    v2 = __fadd_rn(c54, c1);
    if (v2 < b2) { b2 = v2; bp2 = 54u; }
    v = __fadd_rn(c32, c23);
    if (v < b) { b = v; bp = 32u; }
    if (b2 < b) { b = b2; bp = bp2; }
    c55 = __fadd_rn(b, A[55 * 32]);
    P[55 * 32] = (uint8_t)bp;
  }
  float c56;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c16, c40);
    if (v < b) { b = v; bp = 16u; }
    v = __fadd_rn(c32, c24);
    if (v < b) { b = v; bp = 32u; }
    v = __fadd_rn(c48, c8);
    if (v < b) { b = v; bp = 48u; }
    c56 = __fadd_rn(b, A[56 * 32]);
    P[56 * 32] = (uint8_t)bp;
  }
  float c57;
  {
    float b = kTlInf, b2 = kTlInf, v, v2;
    uint32_t bp = 0xffu, bp2 = 0xffu;
    v = __fadd_rn(c8, c49);
    if (v < b) { b = v; bp = 8u; }
    v2 = __fadd_rn(c40, c17);
    if (v2 < b2) { b2 = v2; bp2 = 40u; }
    v = __fadd_rn(c16, c41);
    if (v < b) { b = v; bp = 16u; }
    v2 = __fadd_rn(c48, c9);
    if (v2 < b2) { b2 = v2; bp2 = 48u; }
    v = __fadd_rn(c24, c33);
    if (v < b) { b = v; bp = 24u; }
    v2 = __fadd_rn(c56, c1);
    if (v2 < b2) { b2 = v2; bp2 = 56u; }
    v = __fadd_rn(c32, c25);
    if (v < b) { b = v; bp = 32u; }
    if (b2 < b) { b = b2; bp = bp2; }
    c57 = __fadd_rn(b, A[57 * 32]);
    P[57 * 32] = (uint8_t)bp;
  }
  float c58;
  {
    float b = kTlInf, b2 = kTlInf, v, v2;
    uint32_t bp = 0xffu, bp2 = 0xffu;
    v = __fadd_rn(c8, c50);
    if (v < b) { b = v; bp = 8u; }
    v2 = __fadd_rn(c40, c18);
    if (v2 < b2) { b2 = v2; bp2 = 40u; }
    v = __fadd_rn(c16, c42);
    if (v < b) { b = v; bp = 16u; }
    v2 = __fadd_rn(c48, c10);
    if (v2 < b2) { b2 = v2; bp2 = 48u; }
    v = __fadd_rn(c24, c34);
    if (v < b) { b = v; bp = 24u; }
    v2 = __fadd_rn(c56, c2);
    if (v2 < b2) { b2 = v2; bp2 = 56u; }
    v = __fadd_rn(c32, c26);
    if (v < b) { b = v; bp = 32u; }
    if (b2 < b) { b = b2; bp = bp2; }
    c58 = __fadd_rn(b, A[58 * 32]);
    P[58 * 32] = (uint8_t)bp;
  }
  float c59;
  {
    float b = kTlInf, b2 = kTlInf, v, v2;
    uint32_t bp = 0xffu, bp2 = 0xffu;
    v = __fadd_rn(c2, c57);
    if (v < b) { b = v; bp = 2u; }
    v2 = __fadd_rn(c34, c25);
    if (v2 < b2) { b2 = v2; bp2 = 34u; }
    v = __fadd_rn(c8, c51);
    if (v < b) { b = v; bp = 8u; }
    v2 = __fadd_rn(c40, c19);
    if (v2 < b2) { b2 = v2; bp2 = 40u; }
    v = __fadd_rn(c10, c49);
    if (v < b) { b = v; bp = 10u; }
    v2 = __fadd_rn(c42, c17);
    if (v2 < b2) { b2 = v2; bp2 = 42u; }
    v = __fadd_rn(c16, c43);
    if (v < b) { b = v; bp = 16u; }
    v2 = __fadd_rn(c48, c11);
    if (v2 < b2) { b2 = v2; bp2 = 48u; }
    v = __fadd_rn(c18, c41);
    if (v < b) { b = v; bp = 18u; }
    v2 = __fadd_rn(c50, c9);
    if (v2 < b2) { b2 = v2; bp2 = 50u; }
    v = __fadd_rn(c24, c35);
    if (v < b) { b = v; bp = 24u; }
    v2 = __fadd_rn(c56, c3);
    if (v2 < b2) { b2 = v2; bp2 = 56u; }
    v = __fadd_rn(c26, c33);
    if (v < b) { b = v; bp = 26u; }
    v2 = __fadd_rn(c58, c1);
    if (v2 < b2) { b2 = v2; bp2 = 58u; }
    v = __fadd_rn(c32, c27);
    if (v < b) { b = v; bp = 32u; }
    if (b2 < b) { b = b2; bp = bp2; }
    c59 = __fadd_rn(b, A[59 * 32]);
    P[59 * 32] = (uint8_t)bp;
  }
  float c60;
  {
    float b = kTlInf, b2 = kTlInf, v, v2;
    uint32_t bp = 0xffu, bp2 = 0xffu;
    v = __fadd_rn(c8, c52);
    if (v < b) { b = v; bp = 8u; }
    v2 = __fadd_rn(c40, c20);
    if (v2 < b2) { b2 = v2; bp2 = 40u; }
    v = __fadd_rn(c16, c44);
    if (v < b) { b = v; bp = 16u; }
    v2 = __fadd_rn(c48, c12);
    if (v2 < b2) { b2 = v2; bp2 = 48u; }
    v = __fadd_rn(c24, c36);
    if (v < b) { b = v; bp = 24u; }
    v2 = __fadd_rn(c56, c4);
    if (v2 < b2) { b2 = v2; bp2 = 56u; }
    v = __fadd_rn(c32, c28);
    if (v < b) { b = v; bp = 32u; }
    if (b2 < b) { b = b2; bp = bp2; }
    c60 = __fadd_rn(b, A[60 * 32]);
    P[60 * 32] = (uint8_t)bp;
  }
  float c61;
  {
    float b = kTlInf, b2 = kTlInf, v, v2;
    uint32_t bp = 0xffu, bp2 = 0xffu;
    v = __fadd_rn(c4, c57);
    if (v < b) { b = v; bp = 4u; }
    v2 = __fadd_rn(c36, c25);
    if (v2 < b2) { b2 = v2; bp2 = 36u; }
    v = __fadd_rn(c8, c53);
    if (v < b) { b = v; bp = 8u; }
    v2 = __fadd_rn(c40, c21);
    if (v2 < b2) { b2 = v2; bp2 = 40u; }
    v = __fadd_rn(c12, c49);
    if (v < b) { b = v; bp = 12u; }
    v2 = __fadd_rn(c44, c17);
    if (v2 < b2) { b2 = v2; bp2 = 44u; }
    v = __fadd_rn(c16, c45);
    if (v < b) { b = v; bp = 16u; }
    v2 = __fadd_rn(c48, c13);
    if (v2 < b2) { b2 = v2; bp2 = 48u; }
    v = __fadd_rn(c20, c41);
    if (v < b) { b = v; bp = 20u; }
    v2 = __fadd_rn(c52, c9);
    if (v2 < b2) { b2 = v2; bp2 = 52u; }
    v = __fadd_rn(c24, c37);
    if (v < b) { b = v; bp = 24u; }
    v2 = __fadd_rn(c56, c5);
    if (v2 < b2) { b2 = v2; bp2 = 56u; }
    v = __fadd_rn(c28, c33);
    if (v < b) { b = v; bp = 28u; }
    v2 = __fadd_rn(c60, c1);
    if (v2 < b2) { b2 = v2; bp2 = 60u; }
    v = __fadd_rn(c32, c29);
    if (v < b) { b = v; bp = 32u; }
    if (b2 < b) { b = b2; bp = bp2; }
    c61 = __fadd_rn(b, A[61 * 32]);
    P[61 * 32] = (uint8_t)bp;
  }
  float c62;
  {
    float b = kTlInf, b2 = kTlInf, v, v2;
    uint32_t bp = 0xffu, bp2 = 0xffu;
    v = __fadd_rn(c4, c58);
    if (v < b) { b = v; bp = 4u; }
    v2 = __fadd_rn(c36, c26);
    if (v2 < b2) { b2 = v2; bp2 = 36u; }
    v = __fadd_rn(c8, c54);
    if (v < b) { b = v; bp = 8u; }
    v2 = __fadd_rn(c40, c22);
    if (v2 < b2) { b2 = v2; bp2 = 40u; }
    v = __fadd_rn(c12, c50);
    if (v < b) { b = v; bp = 12u; }
    v2 = __fadd_rn(c44, c18);
    if (v2 < b2) { b2 = v2; bp2 = 44u; }
    v = __fadd_rn(c16, c46);
    if (v < b) { b = v; bp = 16u; }
    v2 = __fadd_rn(c48, c14);
    if (v2 < b2) { b2 = v2; bp2 = 48u; }
    v = __fadd_rn(c20, c42);
    if (v < b) { b = v; bp = 20u; }
    v2 = __fadd_rn(c52, c10);
    if (v2 < b2) { b2 = v2; bp2 = 52u; }
    v = __fadd_rn(c24, c38);
    if (v < b) { b = v; bp = 24u; }
    v2 = __fadd_rn(c56, c6);
    if (v2 < b2) { b2 = v2; bp2 = 56u; }
    v = __fadd_rn(c28, c34);
    if (v < b) { b = v; bp = 28u; }
    v2 = __fadd_rn(c60, c2);
    if (v2 < b2) { b2 = v2; bp2 = 60u; }
    v = __fadd_rn(c32, c30);
    if (v < b) { b = v; bp = 32u; }
    if (b2 < b) { b = b2; bp = bp2; }
    c62 = __fadd_rn(b, A[62 * 32]);
    P[62 * 32] = (uint8_t)bp;
  }
  float c63;
  {
    float b = kTlInf, b2 = kTlInf, v, v2;
    uint32_t bp = 0xffu, bp2 = 0xffu;
    v = __fadd_rn(c2, c61);
    if (v < b) { b = v; bp = 2u; }
    v2 = __fadd_rn(c34, c29);
    if (v2 < b2) { b2 = v2; bp2 = 34u; }
    v = __fadd_rn(c4, c59);
    if (v < b) { b = v; bp = 4u; }
    v2 = __fadd_rn(c36, c27);
    if (v2 < b2) { b2 = v2; bp2 = 36u; }
    v = __fadd_rn(c6, c57);
    if (v < b) { b = v; bp = 6u; }
    v2 = __fadd_rn(c38, c25);
    if (v2 < b2) { b2 = v2; bp2 = 38u; }
    v = __fadd_rn(c8, c55);
    if (v < b) { b = v; bp = 8u; }
    v2 = __fadd_rn(c40, c23);
    if (v2 < b2) { b2 = v2; bp2 = 40u; }
    v = __fadd_rn(c10, c53);
    if (v < b) { b = v; bp = 10u; }
    v2 = __fadd_rn(c42, c21);
    if (v2 < b2) { b2 = v2; bp2 = 42u; }
    v = __fadd_rn(c12, c51);
    if (v < b) { b = v; bp = 12u; }
    v2 = __fadd_rn(c44, c19);
    if (v2 < b2) { b2 = v2; bp2 = 44u; }
    v = __fadd_rn(c14, c49);
    if (v < b) { b = v; bp = 14u; }
    v2 = __fadd_rn(c46, c17);
    if (v2 < b2) { b2 = v2; bp2 = 46u; }
    v = __fadd_rn(c16, c47);
    if (v < b) { b = v; bp = 16u; }
    v2 = __fadd_rn(c48, c15);
    if (v2 < b2) { b2 = v2; bp2 = 48u; }
    v = __fadd_rn(c18, c45);
    if (v < b) { b = v; bp = 18u; }
    v2 = __fadd_rn(c50, c13);
    if (v2 < b2) { b2 = v2; bp2 = 50u; }
    v = __fadd_rn(c20, c43);
    if (v < b) { b = v; bp = 20u; }
    v2 = __fadd_rn(c52, c11);
    if (v2 < b2) { b2 = v2; bp2 = 52u; }
    v = __fadd_rn(c22, c41);
    if (v < b) { b = v; bp = 22u; }
    v2 = __fadd_rn(c54, c9);
    if (v2 < b2) { b2 = v2; bp2 = 54u; }
    v = __fadd_rn(c24, c39);
    if (v < b) { b = v; bp = 24u; }
    v2 = __fadd_rn(c56, c7);
    if (v2 < b2) { b2 = v2; bp2 = 56u; }
    v = __fadd_rn(c26, c37);
    if (v < b) { b = v; bp = 26u; }
    v2 = __fadd_rn(c58, c5);
    if (v2 < b2) { b2 = v2; bp2 = 58u; }
    v = __fadd_rn(c28, c35);
    if (v < b) { b = v; bp = 28u; }
    v2 = __fadd_rn(c60, c3);
    if (v2 < b2) { b2 = v2; bp2 = 60u; }
    v = __fadd_rn(c30, c33);
    if (v < b) { b = v; bp = 30u; }
    v2 = __fadd_rn(c62, c1);
    if (v2 < b2) { b2 = v2; bp2 = 62u; }
    v = __fadd_rn(c32, c31);
    if (v < b) { b = v; bp = 32u; }
    if (b2 < b) { b = b2; bp = bp2; }
    c63 = __fadd_rn(b, A[63 * 32]);
    P[63 * 32] = (uint8_t)bp;
  }
  const float c64 = 0.0f;
  float c65;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c64, c1);
    if (v < b) { b = v; bp = 64u; }
    c65 = __fadd_rn(b, A[65 * 32]);
    P[65 * 32] = (uint8_t)bp;
  }
  float c66;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c64, c2);
    if (v < b) { b = v; bp = 64u; }
    c66 = __fadd_rn(b, A[66 * 32]);
    P[66 * 32] = (uint8_t)bp;
  }
  float c67;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c2, c65);
    if (v < b) { b = v; bp = 2u; }
    v = __fadd_rn(c64, c3);
    if (v < b) { b = v; bp = 64u; }
    v = __fadd_rn(c66, c1);
    if (v < b) { b = v; bp = 66u; }
    c67 = __fadd_rn(b, A[67 * 32]);
    P[67 * 32] = (uint8_t)bp;
  }
  float c68;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c64, c4);
    if (v < b) { b = v; bp = 64u; }
    c68 = __fadd_rn(b, A[68 * 32]);
    P[68 * 32] = (uint8_t)bp;
  }
  float c69;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c4, c65);
    if (v < b) { b = v; bp = 4u; }
    v = __fadd_rn(c64, c5);
    if (v < b) { b = v; bp = 64u; }
    v = __fadd_rn(c68, c1);
    if (v < b) { b = v; bp = 68u; }
    c69 = __fadd_rn(b, A[69 * 32]);
    P[69 * 32] = (uint8_t)bp;
  }
  float c70;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c4, c66);
    if (v < b) { b = v; bp = 4u; }
    v = __fadd_rn(c64, c6);
    if (v < b) { b = v; bp = 64u; }
    v = __fadd_rn(c68, c2);
    if (v < b) { b = v; bp = 68u; }
    c70 = __fadd_rn(b, A[70 * 32]);
    P[70 * 32] = (uint8_t)bp;
  }
  float c71;
  {
    float b = kTlInf, b2 = kTlInf, v, v2;
    uint32_t bp = 0xffu, bp2 = 0xffu;
    v = __fadd_rn(c2, c69);
    if (v < b) { b = v; bp = 2u; }
    v2 = __fadd_rn(c66, c5);
    if (v2 < b2) { b2 = v2; bp2 = 66u; }
    v = __fadd_rn(c4, c67);
    if (v < b) { b = v; bp = 4u; }
    v2 = __fadd_rn(c68, c3);
    if (v2 < b2) { b2 = v2; bp2 = 68u; }
    v = __fadd_rn(c6, c65);
    if (v < b) { b = v; bp = 6u; }
    v2 = __fadd_rn(c70, c1);
    if (v2 < b2) { b2 = v2; bp2 = 70u; }
    v = __fadd_rn(c64, c7);
    if (v < b) { b = v; bp = 64u; }
    if (b2 < b) { b = b2; bp = bp2; }
    c71 = __fadd_rn(b, A[71 * 32]);
    P[71 * 32] = (uint8_t)bp;
  }
  float c72;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c64, c8);
    if (v < b) { b = v; bp = 64u; }
    c72 = __fadd_rn(b, A[72 * 32]);
    P[72 * 32] = (uint8_t)bp;
  }
  float c73;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c8, c65);
    if (v < b) { b = v; bp = 8u; }
    v = __fadd_rn(c64, c9);
    if (v < b) { b = v; bp = 64u; }
    v = __fadd_rn(c72, c1);
    if (v < b) { b = v; bp = 72u; }
    c73 = __fadd_rn(b, A[73 * 32]);
    P[73 * 32] = (uint8_t)bp;
  }
  float c74;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c8, c66);
    if (v < b) { b = v; bp = 8u; }
    v = __fadd_rn(c64, c10);
    if (v < b) { b = v; bp = 64u; }
    v = __fadd_rn(c72, c2);
    if (v < b) { b = v; bp = 72u; }
    c74 = __fadd_rn(b, A[74 * 32]);
    P[74 * 32] = (uint8_t)bp;
  }
  float c75;
  {
    float b = kTlInf, b2 = kTlInf, v, v2;
    uint32_t bp = 0xffu, bp2 = 0xffu;
    v = __fadd_rn(c2, c73);
    if (v < b) { b = v; bp = 2u; }
    v2 = __fadd_rn(c66, c9);
    if (v2 < b2) { b2 = v2; bp2 = 66u; }
    v = __fadd_rn(c8, c67);
    if (v < b) { b = v; bp = 8u; }
    v2 = __fadd_rn(c72, c3);
    if (v2 < b2) { b2 = v2; bp2 = 72u; }
    v = __fadd_rn(c10, c65);
    if (v < b) { b = v; bp = 10u; }
    v2 = __fadd_rn(c74, c1);
    if (v2 < b2) { b2 = v2; bp2 = 74u; }
    v = __fadd_rn(c64, c11);
    if (v < b) { b = v; bp = 64u; }
    if (b2 < b) { b = b2; bp = bp2; }
    c75 = __fadd_rn(b, A[75 * 32]);
    P[75 * 32] = (uint8_t)bp;
  }
  float c76;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c8, c68);
    if (v < b) { b = v; bp = 8u; }
    v = __fadd_rn(c64, c12);
    if (v < b) { b = v; bp = 64u; }
    v = __fadd_rn(c72, c4);
    if (v < b) { b = v; bp = 72u; }
    c76 = __fadd_rn(b, A[76 * 32]);
    P[76 * 32] = (uint8_t)bp;
  }
  float c77;
  {
    float b = kTlInf, b2 = kTlInf, v, v2;
    uint32_t bp = 0xffu, bp2 = 0xffu;
    v = __fadd_rn(c4, c73);
    if (v < b) { b = v; bp = 4u; }
    v2 = __fadd_rn(c68, c9);
    if (v2 < b2) { b2 = v2; bp2 = 68u; }
    v = __fadd_rn(c8, c69);
    if (v < b) { b = v; bp = 8u; }
    v2 = __fadd_rn(c72, c5);
    if (v2 < b2) { b2 = v2; bp2 = 72u; }
    v = __fadd_rn(c12, c65);
    if (v < b) { b = v; bp = 12u; }
    v2 = __fadd_rn(c76, c1);
    if (v2 < b2) { b2 = v2; bp2 = 76u; }
    v = __fadd_rn(c64, c13);
    if (v < b) { b = v; bp = 64u; }
    if (b2 < b) { b = b2; bp = bp2; }
    c77 = __fadd_rn(b, A[77 * 32]);
    P[77 * 32] = (uint8_t)bp;
  }
  float c78;
  {
    float b = kTlInf, b2 = kTlInf, v, v2;
    uint32_t bp = 0xffu, bp2 = 0xffu;
    v = __fadd_rn(c4, c74);
    if (v < b) { b = v; bp = 4u; }
    v2 = __fadd_rn(c68, c10);
    if (v2 < b2) { b2 = v2; bp2 = 68u; }
    v = __fadd_rn(c8, c70);
    if (v < b) { b = v; bp = 8u; }
    v2 = __fadd_rn(c72, c6);
    if (v2 < b2) { b2 = v2; bp2 = 72u; }
    v = __fadd_rn(c12, c66);
    if (v < b) { b = v; bp = 12u; }
    v2 = __fadd_rn(c76, c2);
    if (v2 < b2) { b2 = v2; bp2 = 76u; }
    v = __fadd_rn(c64, c14);
    if (v < b) { b = v; bp = 64u; }
    if (b2 < b) { b = b2; bp = bp2; }
    c78 = __fadd_rn(b, A[78 * 32]);
    P[78 * 32] = (uint8_t)bp;
  }
  float c79;
  {
    float b = kTlInf, b2 = kTlInf, v, v2;
    uint32_t bp = 0xffu, bp2 = 0xffu;
    v = __fadd_rn(c2, c77);
    if (v < b) { b = v; bp = 2u; }
    v2 = __fadd_rn(c66, c13);
    if (v2 < b2) { b2 = v2; bp2 = 66u; }
    v = __fadd_rn(c4, c75);
    if (v < b) { b = v; bp = 4u; }
    v2 = __fadd_rn(c68, c11);
    if (v2 < b2) { b2 = v2; bp2 = 68u; }
    v = __fadd_rn(c6, c73);
    if (v < b) { b = v; bp = 6u; }
    v2 = __fadd_rn(c70, c9);
    if (v2 < b2) { b2 = v2; bp2 = 70u; }
    v = __fadd_rn(c8, c71);
    if (v < b) { b = v; bp = 8u; }
    v2 = __fadd_rn(c72, c7);
    if (v2 < b2) { b2 = v2; bp2 = 72u; }
    v = __fadd_rn(c10, c69);
    if (v < b) { b = v; bp = 10u; }
    v2 = __fadd_rn(c74, c5);
    if (v2 < b2) { b2 = v2; bp2 = 74u; }
    v = __fadd_rn(c12, c67);
    if (v < b) { b = v; bp = 12u; }
    v2 = __fadd_rn(c76, c3);
    if (v2 < b2) { b2 = v2; bp2 = 76u; }
    v = __fadd_rn(c14, c65);
    if (v < b) { b = v; bp = 14u; }
    v2 = __fadd_rn(c78, c1);
    if (v2 < b2) { b2 = v2; bp2 = 78u; }
    v = __fadd_rn(c64, c15);
    if (v < b) { b = v; bp = 64u; }
    if (b2 < b) { b = b2; bp = bp2; }
    c79 = __fadd_rn(b, A[79 * 32]);
    P[79 * 32] = (uint8_t)bp;
  }
  float c80;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c64, c16);
    if (v < b) { b = v; bp = 64u; }
    c80 = __fadd_rn(b, A[80 * 32]);
    P[80 * 32] = (uint8_t)bp;
  }
  float c81;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c16, c65);
    if (v < b) { b = v; bp = 16u; }
    v = __fadd_rn(c64, c17);
    if (v < b) { b = v; bp = 64u; }
    v = __fadd_rn(c80, c1);
    if (v < b) { b = v; bp = 80u; }
    c81 = __fadd_rn(b, A[81 * 32]);
    P[81 * 32] = (uint8_t)bp;
  }
  float c82;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c16, c66);
    if (v < b) { b = v; bp = 16u; }
    v = __fadd_rn(c64, c18);
    if (v < b) { b = v; bp = 64u; }
    v = __fadd_rn(c80, c2);
    if (v < b) { b = v; bp = 80u; }
    c82 = __fadd_rn(b, A[82 * 32]);
    P[82 * 32] = (uint8_t)bp;
  }
  float c83;
  {
    float b = kTlInf, b2 = kTlInf, v, v2;
    uint32_t bp = 0xffu, bp2 = 0xffu;
    v = __fadd_rn(c2, c81);
    if (v < b) { b = v; bp = 2u; }
    v2 = __fadd_rn(c66, c17);
    if (v2 < b2) { b2 = v2; bp2 = 66u; }
    v = __fadd_rn(c16, c67);
    if (v < b) { b = v; bp = 16u; }
    v2 = __fadd_rn(c80, c3);
    if (v2 < b2) { b2 = v2; bp2 = 80u; }
    v = __fadd_rn(c18, c65);
    if (v < b) { b = v; bp = 18u; }
    v2 = __fadd_rn(c82, c1);
    if (v2 < b2) { b2 = v2; bp2 = 82u; }
    v = __fadd_rn(c64, c19);
    if (v < b) { b = v; bp = 64u; }
    if (b2 < b) { b = b2; bp = bp2; }
    c83 = __fadd_rn(b, A[83 * 32]);
    P[83 * 32] = (uint8_t)bp;
  }
  float c84;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c16, c68);
    if (v < b) { b = v; bp = 16u; }
    v = __fadd_rn(c64, c20);
    if (v < b) { b = v; bp = 64u; }
    v = __fadd_rn(c80, c4);
    if (v < b) { b = v; bp = 80u; }
    c84 = __fadd_rn(b, A[84 * 32]);
    P[84 * 32] = (uint8_t)bp;
  }
  float c85;
  {
    float b = kTlInf, b2 = kTlInf, v, v2;
    uint32_t bp = 0xffu, bp2 = 0xffu;
    v = __fadd_rn(c4, c81);
    if (v < b) { b = v; bp = 4u; }
    v2 = __fadd_rn(c68, c17);
    if (v2 < b2) { b2 = v2; bp2 = 68u; }
    v = __fadd_rn(c16, c69);
    if (v < b) { b = v; bp = 16u; }
    v2 = __fadd_rn(c80, c5);
    if (v2 < b2) { b2 = v2; bp2 = 80u; }
    v = __fadd_rn(c20, c65);
    if (v < b) { b = v; bp = 20u; }
    v2 = __fadd_rn(c84, c1);
    if (v2 < b2) { b2 = v2; bp2 = 84u; }
    v = __fadd_rn(c64, c21);
    if (v < b) { b = v; bp = 64u; }
    if (b2 < b) { b = b2; bp = bp2; }
    c85 = __fadd_rn(b, A[85 * 32]);
    P[85 * 32] = (uint8_t)bp;
  }
  float c86;
  {
    float b = kTlInf, b2 = kTlInf, v, v2;
    uint32_t bp = 0xffu, bp2 = 0xffu;
    v = __fadd_rn(c4, c82);
    if (v < b) { b = v; bp = 4u; }
    v2 = __fadd_rn(c68, c18);
    if (v2 < b2) { b2 = v2; bp2 = 68u; }
    v = __fadd_rn(c16, c70);
    if (v < b) { b = v; bp = 16u; }
    v2 = __fadd_rn(c80, c6);
    if (v2 < b2) { b2 = v2; bp2 = 80u; }
    v = __fadd_rn(c20, c66);
    if (v < b) { b = v; bp = 20u; }
    v2 = __fadd_rn(c84, c2);
    if (v2 < b2) { b2 = v2; bp2 = 84u; }
    v = __fadd_rn(c64, c22);
    if (v < b) { b = v; bp = 64u; }
    if (b2 < b) { b = b2; bp = bp2; }
    c86 = __fadd_rn(b, A[86 * 32]);
    P[86 * 32] = (uint8_t)bp;
  }
  float c87;
  {
    float b = kTlInf, b2 = kTlInf, v, v2;
    uint32_t bp = 0xffu, bp2 = 0xffu;
    v = __fadd_rn(c2, c85);
    if (v < b) { b = v; bp = 2u; }
    v2 = __fadd_rn(c66, c21);
    if (v2 < b2) { b2 = v2; bp2 = 66u; }
    v = __fadd_rn(c4, c83);
    if (v < b) { b = v; bp = 4u; }
    v2 = __fadd_rn(c68, c19);
    if (v2 < b2) { b2 = v2; bp2 = 68u; }
    v = __fadd_rn(c6, c81);
    if (v < b) { b = v; bp = 6u; }
    v2 = __fadd_rn(c70, c17);
    if (v2 < b2) { b2 = v2; bp2 = 70u; }
    v = __fadd_rn(c16, c71);
    if (v < b) { b = v; bp = 16u; }
    v2 = __fadd_rn(c80, c7);
    if (v2 < b2) { b2 = v2; bp2 = 80u; }
    v = __fadd_rn(c18, c69);
    if (v < b) { b = v; bp = 18u; }
    v2 = __fadd_rn(c82, c5);
    if (v2 < b2) { b2 = v2; bp2 = 82u; }
    v = __fadd_rn(c20, c67);
    if (v < b) { b = v; bp = 20u; }
    v2 = __fadd_rn(c84, c3);
    if (v2 < b2) { b2 = v2; bp2 = 84u; }
    v = __fadd_rn(c22, c65);
    if (v < b) { b = v; bp = 22u; }
    v2 = __fadd_rn(c86, c1);
    if (v2 < b2) { b2 = v2; bp2 = 86u; }
    v = __fadd_rn(c64, c23);
    if (v < b) { b = v; bp = 64u; }
    if (b2 < b) { b = b2; bp = bp2; }
    c87 = __fadd_rn(b, A[87 * 32]);
    P[87 * 32] = (uint8_t)bp;
  }
  float c88;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c16, c72);
    if (v < b) { b = v; bp = 16u; }
    v = __fadd_rn(c64, c24);
    if (v < b) { b = v; bp = 64u; }
    v = __fadd_rn(c80, c8);
    if (v < b) { b = v; bp = 80u; }
    c88 = __fadd_rn(b, A[88 * 32]);
    P[88 * 32] = (uint8_t)bp;
  }
  float c89;
  {
    float b = kTlInf, b2 = kTlInf, v, v2;
    uint32_t bp = 0xffu, bp2 = 0xffu;
    v = __fadd_rn(c8, c81);
    if (v < b) { b = v; bp = 8u; }
    v2 = __fadd_rn(c72, c17);
    if (v2 < b2) { b2 = v2; bp2 = 72u; }
    v = __fadd_rn(c16, c73);
    if (v < b) { b = v; bp = 16u; }
    v2 = __fadd_rn(c80, c9);
    if (v2 < b2) { b2 = v2; bp2 = 80u; }
    v = __fadd_rn(c24, c65);
    if (v < b) { b = v; bp = 24u; }
    v2 = __fadd_rn(c88, c1);
    if (v2 < b2) { b2 = v2; bp2 = 88u; }
    v = __fadd_rn(c64, c25);
    if (v < b) { b = v; bp = 64u; }
    if (b2 < b) { b = b2; bp = bp2; }
    c89 = __fadd_rn(b, A[89 * 32]);
    P[89 * 32] = (uint8_t)bp;
  }
  float c90;
  {
    float b = kTlInf, b2 = kTlInf, v, v2;
    uint32_t bp = 0xffu, bp2 = 0xffu;
    v = __fadd_rn(c8, c82);
    if (v < b) { b = v; bp = 8u; }
    v2 = __fadd_rn(c72, c18);
    if (v2 < b2) { b2 = v2; bp2 = 72u; }
    v = __fadd_rn(c16, c74);
    if (v < b) { b = v; bp = 16u; }
    v2 = __fadd_rn(c80, c10);
    if (v2 < b2) { b2 = v2; bp2 = 80u; }
    v = __fadd_rn(c24, c66);
    if (v < b) { b = v; bp = 24u; }
    v2 = __fadd_rn(c88, c2);
    if (v2 < b2) { b2 = v2; bp2 = 88u; }
    v = __fadd_rn(c64, c26);
    if (v < b) { b = v; bp = 64u; }
    if (b2 < b) { b = b2; bp = bp2; }
    c90 = __fadd_rn(b, A[90 * 32]);
    P[90 * 32] = (uint8_t)bp;
  }
  float c91;
  {
    float b = kTlInf, b2 = kTlInf, v, v2;
    uint32_t bp = 0xffu, bp2 = 0xffu;
    v = __fadd_rn(c2, c89);
    if (v < b) { b = v; bp = 2u; }
    v2 = __fadd_rn(c66, c25);
    if (v2 < b2) { b2 = v2; bp2 = 66u; }
    v = __fadd_rn(c8, c83);
    if (v < b) { b = v; bp = 8u; }
    v2 = __fadd_rn(c72, c19);
    if (v2 < b2) { b2 = v2; bp2 = 72u; }
    v = __fadd_rn(c10, c81);
    if (v < b) { b = v; bp = 10u; }
    v2 = __fadd_rn(c74, c17);
    if (v2 < b2) { b2 = v2; bp2 = 74u; }
    v = __fadd_rn(c16, c75);
    if (v < b) { b = v; bp = 16u; }
    v2 = __fadd_rn(c80, c11);
    if (v2 < b2) { b2 = v2; bp2 = 80u; }
    v = __fadd_rn(c18, c73);
    if (v < b) { b = v; bp = 18u; }
    v2 = __fadd_rn(c82, c9);
    if (v2 < b2) { b2 = v2; bp2 = 82u; }
    v = __fadd_rn(c24, c67);
    if (v < b) { b = v; bp = 24u; }
    v2 = __fadd_rn(c88, c3);
    if (v2 < b2) { b2 = v2; bp2 = 88u; }
    v = __fadd_rn(c26, c65);
    if (v < b) { b = v; bp = 26u; }
    v2 = __fadd_rn(c90, c1);
    if (v2 < b2) { b2 = v2; bp2 = 90u; }
    v = __fadd_rn(c64, c27);
    if (v < b) { b = v; bp = 64u; }
    if (b2 < b) { b = b2; bp = bp2; }
    c91 = __fadd_rn(b, A[91 * 32]);
    P[91 * 32] = (uint8_t)bp;
  }
  float c92;
  {
    float b = kTlInf, b2 = kTlInf, v, v2;
    uint32_t bp = 0xffu, bp2 = 0xffu;
    v = __fadd_rn(c8, c84);
    if (v < b) { b = v; bp = 8u; }
    v2 = __fadd_rn(c72, c20);
    if (v2 < b2) { b2 = v2; bp2 = 72u; }
    v = __fadd_rn(c16, c76);
    if (v < b) { b = v; bp = 16u; }
    v2 = __fadd_rn(c80, c12);
    if (v2 < b2) { b2 = v2; bp2 = 80u; }
    v = __fadd_rn(c24, c68);
    if (v < b) { b = v; bp = 24u; }
    v2 = __fadd_rn(c88, c4);
    if (v2 < b2) { b2 = v2; bp2 = 88u; }
    v = __fadd_rn(c64, c28);
    if (v < b) { b = v; bp = 64u; }
    if (b2 < b) { b = b2; bp = bp2; }
    c92 = __fadd_rn(b, A[92 * 32]);
    P[92 * 32] = (uint8_t)bp;
  }
  float c93;
  {
    float b = kTlInf, b2 = kTlInf, v, v2;
    uint32_t bp = 0xffu, bp2 = 0xffu;
    v = __fadd_rn(c4, c89);
    if (v < b) { b = v; bp = 4u; }
    v2 = __fadd_rn(c68, c25);
    if (v2 < b2) { b2 = v2; bp2 = 68u; }
    v = __fadd_rn(c8, c85);
    if (v < b) { b = v; bp = 8u; }
    v2 = __fadd_rn(c72, c21);
    if (v2 < b2) { b2 = v2; bp2 = 72u; }
    v = __fadd_rn(c12, c81);
    if (v < b) { b = v; bp = 12u; }
    v2 = __fadd_rn(c76, c17);
    if (v2 < b2) { b2 = v2; bp2 = 76u; }
    v = __fadd_rn(c16, c77);
    if (v < b) { b = v; bp = 16u; }
    v2 = __fadd_rn(c80, c13);
    if (v2 < b2) { b2 = v2; bp2 = 80u; }
    v = __fadd_rn(c20, c73);
    if (v < b) { b = v; bp = 20u; }
    v2 = __fadd_rn(c84, c9);
    if (v2 < b2) { b2 = v2; bp2 = 84u; }
    v = __fadd_rn(c24, c69);
    if (v < b) { b = v; bp = 24u; }
    v2 = __fadd_rn(c88, c5);
    if (v2 < b2) { b2 = v2; bp2 = 88u; }
    v = __fadd_rn(c28, c65);
    if (v < b) { b = v; bp = 28u; }
    v2 = __fadd_rn(c92, c1);
    if (v2 < b2) { b2 = v2; bp2 = 92u; }
    v = __fadd_rn(c64, c29);
    if (v < b) { b = v; bp = 64u; }
    if (b2 < b) { b = b2; bp = bp2; }
    c93 = __fadd_rn(b, A[93 * 32]);
    P[93 * 32] = (uint8_t)bp;
  }
  float c94;
  {
    float b = kTlInf, b2 = kTlInf, v, v2;
    uint32_t bp = 0xffu, bp2 = 0xffu;
    v = __fadd_rn(c4, c90);
    if (v < b) { b = v; bp = 4u; }
    v2 = __fadd_rn(c68, c26);
    if (v2 < b2) { b2 = v2; bp2 = 68u; }
    v = __fadd_rn(c8, c86);
    if (v < b) { b = v; bp = 8u; }
    v2 = __fadd_rn(c72, c22);
    if (v2 < b2) { b2 = v2; bp2 = 72u; }
    v = __fadd_rn(c12, c82);
    if (v < b) { b = v; bp = 12u; }
    v2 = __fadd_rn(c76, c18);
    if (v2 < b2) { b2 = v2; bp2 = 76u; }
    v = __fadd_rn(c16, c78);
    if (v < b) { b = v; bp = 16u; }
    v2 = __fadd_rn(c80, c14);
    if (v2 < b2) { b2 = v2; bp2 = 80u; }
    v = __fadd_rn(c20, c74);
    if (v < b) { b = v; bp = 20u; }
    v2 = __fadd_rn(c84, c10);
    if (v2 < b2) { b2 = v2; bp2 = 84u; }
    v = __fadd_rn(c24, c70);
    if (v < b) { b = v; bp = 24u; }
    v2 = __fadd_rn(c88, c6);
    if (v2 < b2) { b2 = v2; bp2 = 88u; }
    v = __fadd_rn(c28, c66);
    if (v < b) { b = v; bp = 28u; }
    v2 = __fadd_rn(c92, c2);
    if (v2 < b2) { b2 = v2; bp2 = 92u; }
    v = __fadd_rn(c64, c30);
    if (v < b) { b = v; bp = 64u; }
    if (b2 < b) { b = b2; bp = bp2; }
    c94 = __fadd_rn(b, A[94 * 32]);
    P[94 * 32] = (uint8_t)bp;
  }
  float c95;
  {
    float b = kTlInf, b2 = kTlInf, v, v2;
    uint32_t bp = 0xffu, bp2 = 0xffu;
    v = __fadd_rn(c2, c93);
    if (v < b) { b = v; bp = 2u; }
    v2 = __fadd_rn(c66, c29);
    if (v2 < b2) { b2 = v2; bp2 = 66u; }
    v = __fadd_rn(c4, c91);
    if (v < b) { b = v; bp = 4u; }
    v2 = __fadd_rn(c68, c27);
    if (v2 < b2) { b2 = v2; bp2 = 68u; }
    v = __fadd_rn(c6, c89);
    if (v < b) { b = v; bp = 6u; }
    v2 = __fadd_rn(c70, c25);
    if (v2 < b2) { b2 = v2; bp2 = 70u; }
    v = __fadd_rn(c8, c87);
    if (v < b) { b = v; bp = 8u; }
    v2 = __fadd_rn(c72, c23);
    if (v2 < b2) { b2 = v2; bp2 = 72u; }
    v = __fadd_rn(c10, c85);
    if (v < b) { b = v; bp = 10u; }
    v2 = __fadd_rn(c74, c21);
    if (v2 < b2) { b2 = v2; bp2 = 74u; }
    v = __fadd_rn(c12, c83);
    if (v < b) { b = v; bp = 12u; }
    v2 = __fadd_rn(c76, c19);
    if (v2 < b2) { b2 = v2; bp2 = 76u; }
    v = __fadd_rn(c14, c81);
    if (v < b) { b = v; bp = 14u; }
    v2 = __fadd_rn(c78, c17);
    if (v2 < b2) { b2 = v2; bp2 = 78u; }
    v = __fadd_rn(c16, c79);
    if (v < b) { b = v; bp = 16u; }
    v2 = __fadd_rn(c80, c15);
    if (v2 < b2) { b2 = v2; bp2 = 80u; }
    v = __fadd_rn(c18, c77);
    if (v < b) { b = v; bp = 18u; }
    v2 = __fadd_rn(c82, c13);
    if (v2 < b2) { b2 = v2; bp2 = 82u; }
    v = __fadd_rn(c20, c75);
    if (v < b) { b = v; bp = 20u; }
    v2 = __fadd_rn(c84, c11);
    if (v2 < b2) { b2 = v2; bp2 = 84u; }
    v = __fadd_rn(c22, c73);
    if (v < b) { b = v; bp = 22u; }
    v2 = __fadd_rn(c86, c9);
    if (v2 < b2) { b2 = v2; bp2 = 86u; }
    v = __fadd_rn(c24, c71);
    if (v < b) { b = v; bp = 24u; }
    v2 = __fadd_rn(c88, c7);
    if (v2 < b2) { b2 = v2; bp2 = 88u; }
    v = __fadd_rn(c26, c69);
    if (v < b) { b = v; bp = 26u; }
    v2 = __fadd_rn(c90, c5);
    if (v2 < b2) { b2 = v2; bp2 = 90u; }
    v = __fadd_rn(c28, c67);
    if (v < b) { b = v; bp = 28u; }
    v2 = __fadd_rn(c92, c3);
    if (v2 < b2) { b2 = v2; bp2 = 92u; }
    v = __fadd_rn(c30, c65);
    if (v < b) { b = v; bp = 30u; }
    v2 = __fadd_rn(c94, c1);
    if (v2 < b2) { b2 = v2; bp2 = 94u; }
    v = __fadd_rn(c64, c31);
    if (v < b) { b = v; bp = 64u; }
    if (b2 < b) { b = b2; bp = bp2; }
    c95 = __fadd_rn(b, A[95 * 32]);
    P[95 * 32] = (uint8_t)bp;
  }
  float c96;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c64, c32);
    if (v < b) { b = v; bp = 64u; }
    c96 = __fadd_rn(b, A[96 * 32]);
    P[96 * 32] = (uint8_t)bp;
  }
  float c97;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c32, c65);
    if (v < b) { b = v; bp = 32u; }
    v = __fadd_rn(c64, c33);
    if (v < b) { b = v; bp = 64u; }
    v = __fadd_rn(c96, c1);
    if (v < b) { b = v; bp = 96u; }
    c97 = __fadd_rn(b, A[97 * 32]);
    P[97 * 32] = (uint8_t)bp;
  }
  float c98;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c32, c66);
    if (v < b) { b = v; bp = 32u; }
    v = __fadd_rn(c64, c34);
    if (v < b) { b = v; bp = 64u; }
    v = __fadd_rn(c96, c2);
    if (v < b) { b = v; bp = 96u; }
    c98 = __fadd_rn(b, A[98 * 32]);
    P[98 * 32] = (uint8_t)bp;
  }
  float c99;
  {
    float b = kTlInf, b2 = kTlInf, v, v2;
    uint32_t bp = 0xffu, bp2 = 0xffu;
    v = __fadd_rn(c2, c97);
    if (v < b) { b = v; bp = 2u; }
    v2 = __fadd_rn(c66, c33);
    if (v2 < b2) { b2 = v2; bp2 = 66u; }
    v = __fadd_rn(c32, c67);
    if (v < b) { b = v; bp = 32u; }
    v2 = __fadd_rn(c96, c3);
    if (v2 < b2) { b2 = v2; bp2 = 96u; }
    v = __fadd_rn(c34, c65);
    if (v < b) { b = v; bp = 34u; }
    v2 = __fadd_rn(c98, c1);
    if (v2 < b2) { b2 = v2; bp2 = 98u; }
    v = __fadd_rn(c64, c35);
    if (v < b) { b = v; bp = 64u; }
    if (b2 < b) { b = b2; bp = bp2; }
    c99 = __fadd_rn(b, A[99 * 32]);
    P[99 * 32] = (uint8_t)bp;
  }
  float c100;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c32, c68);
    if (v < b) { b = v; bp = 32u; }
    v = __fadd_rn(c64, c36);
    if (v < b) { b = v; bp = 64u; }
    v = __fadd_rn(c96, c4);
    if (v < b) { b = v; bp = 96u; }
    c100 = __fadd_rn(b, A[100 * 32]);
    P[100 * 32] = (uint8_t)bp;
  }
  float c101;
  {
    float b = kTlInf, b2 = kTlInf, v, v2;
    uint32_t bp = 0xffu, bp2 = 0xffu;
    v = __fadd_rn(c4, c97);
    if (v < b) { b = v; bp = 4u; }
    v2 = __fadd_rn(c68, c33);
    if (v2 < b2) { b2 = v2; bp2 = 68u; }
    v = __fadd_rn(c32, c69);
    if (v < b) { b = v; bp = 32u; }
    v2 = __fadd_rn(c96, c5);
    if (v2 < b2) { b2 = v2; bp2 = 96u; }
    v = __fadd_rn(c36, c65);
    if (v < b) { b = v; bp = 36u; }
    v2 = __fadd_rn(c100, c1);
    if (v2 < b2) { b2 = v2; bp2 = 100u; }
    v = __fadd_rn(c64, c37);
    if (v < b) { b = v; bp = 64u; }
    if (b2 < b) { b = b2; bp = bp2; }
    c101 = __fadd_rn(b, A[101 * 32]);
    P[101 * 32] = (uint8_t)bp;
  }
  float c102;
  {
    float b = kTlInf, b2 = kTlInf, v, v2;
    uint32_t bp = 0xffu, bp2 = 0xffu;
    v = __fadd_rn(c4, c98);
    if (v < b) { b = v; bp = 4u; }
    v2 = __fadd_rn(c68, c34);
    if (v2 < b2) { b2 = v2; bp2 = 68u; }
    v = __fadd_rn(c32, c70);
    if (v < b) { b = v; bp = 32u; }
    v2 = __fadd_rn(c96, c6);
    if (v2 < b2) { b2 = v2; bp2 = 96u; }
    v = __fadd_rn(c36, c66);
    if (v < b) { b = v; bp = 36u; }
    v2 = __fadd_rn(c100, c2);
    if (v2 < b2) { b2 = v2; bp2 = 100u; }
    v = __fadd_rn(c64, c38);
    if (v < b) { b = v; bp = 64u; }
    if (b2 < b) { b = b2; bp = bp2; }
    c102 = __fadd_rn(b, A[102 * 32]);
    P[102 * 32] = (uint8_t)bp;
  }
  float c103;
  {
    float b = kTlInf, b2 = kTlInf, v, v2;
    uint32_t bp = 0xffu, bp2 = 0xffu;
    v = __fadd_rn(c2, c101);
    if (v < b) { b = v; bp = 2u; }
    v2 = __fadd_rn(c66, c37);
    if (v2 < b2) { b2 = v2; bp2 = 66u; }
    v = __fadd_rn(c4, c99);
    if (v < b) { b = v; bp = 4u; }
    v2 = __fadd_rn(c68, c35);
    if (v2 < b2) { b2 = v2; bp2 = 68u; }
    v = __fadd_rn(c6, c97);
    if (v < b) { b = v; bp = 6u; }
    v2 = __fadd_rn(c70, c33);
    if (v2 < b2) { b2 = v2; bp2 = 70u; }
    v = __fadd_rn(c32, c71);
    if (v < b) { b = v; bp = 32u; }
    v2 = __fadd_rn(c96, c7);
    if (v2 < b2) { b2 = v2; bp2 = 96u; }
    v = __fadd_rn(c34, c69);
    if (v < b) { b = v; bp = 34u; }
    v2 = __fadd_rn(c98, c5);
    if (v2 < b2) { b2 = v2; bp2 = 98u; }
    v = __fadd_rn(c36, c67);
    if (v < b) { b = v; bp = 36u; }
    v2 = __fadd_rn(c100, c3);
    if (v2 < b2) { b2 = v2; bp2 = 100u; }
    v = __fadd_rn(c38, c65);
    if (v < b) { b = v; bp = 38u; }
    v2 = __fadd_rn(c102, c1);
    if (v2 < b2) { b2 = v2; bp2 = 102u; }
    v = __fadd_rn(c64, c39);
    if (v < b) { b = v; bp = 64u; }
    if (b2 < b) { b = b2; bp = bp2; }
    c103 = __fadd_rn(b, A[103 * 32]);
    P[103 * 32] = (uint8_t)bp;
  }
  float c104;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c32, c72);
    if (v < b) { b = v; bp = 32u; }
    v = __fadd_rn(c64, c40);
    if (v < b) { b = v; bp = 64u; }
    v = __fadd_rn(c96, c8);
    if (v < b) { b = v; bp = 96u; }
    c104 = __fadd_rn(b, A[104 * 32]);
    P[104 * 32] = (uint8_t)bp;
  }
  float c105;
  {
    float b = kTlInf, b2 = kTlInf, v, v2;
    uint32_t bp = 0xffu, bp2 = 0xffu;
    v = __fadd_rn(c8, c97);
    if (v < b) { b = v; bp = 8u; }
    v2 = __fadd_rn(c72, c33);
    if (v2 < b2) { b2 = v2; bp2 = 72u; }
    v = __fadd_rn(c32, c73);
    if (v < b) { b = v; bp = 32u; }
    v2 = __fadd_rn(c96, c9);
    if (v2 < b2) { b2 = v2; bp2 = 96u; }
    v = __fadd_rn(c40, c65);
    if (v < b) { b = v; bp = 40u; }
    v2 = __fadd_rn(c104, c1);
    if (v2 < b2) { b2 = v2; bp2 = 104u; }
    v = __fadd_rn(c64, c41);
    if (v < b) { b = v; bp = 64u; }
    if (b2 < b) { b = b2; bp = bp2; }
    c105 = __fadd_rn(b, A[105 * 32]);
    P[105 * 32] = (uint8_t)bp;
  }
  float c106;
  {
    float b = kTlInf, b2 = kTlInf, v, v2;
    uint32_t bp = 0xffu, bp2 = 0xffu;
    v = __fadd_rn(c8, c98);
    if (v < b) { b = v; bp = 8u; }
    v2 = __fadd_rn(c72, c34);
    if (v2 < b2) { b2 = v2; bp2 = 72u; }
    v = __fadd_rn(c32, c74);
    if (v < b) { b = v; bp = 32u; }
    v2 = __fadd_rn(c96, c10);
    if (v2 < b2) { b2 = v2; bp2 = 96u; }
    v = __fadd_rn(c40, c66);
    if (v < b) { b = v; bp = 40u; }
    v2 = __fadd_rn(c104, c2);
    if (v2 < b2) { b2 = v2; bp2 = 104u; }
    v = __fadd_rn(c64, c42);
    if (v < b) { b = v; bp = 64u; }
    if (b2 < b) { b = b2; bp = bp2; }
    c106 = __fadd_rn(b, A[106 * 32]);
    P[106 * 32] = (uint8_t)bp;
  }
  float c107;
  {
    float b = kTlInf, b2 = kTlInf, v, v2;
    uint32_t bp = 0xffu, bp2 = 0xffu;
    v = __fadd_rn(c2, c105);
    if (v < b) { b = v; bp = 2u; }
    v2 = __fadd_rn(c66, c41);
    if (v2 < b2) { b2 = v2; bp2 = 66u; }
    v = __fadd_rn(c8, c99);
    if (v < b) { b = v; bp = 8u; }
    v2 = __fadd_rn(c72, c35);
    if (v2 < b2) { b2 = v2; bp2 = 72u; }
    v = __fadd_rn(c10, c97);
    if (v < b) { b = v; bp = 10u; }
    v2 = __fadd_rn(c74, c33);
    if (v2 < b2) { b2 = v2; bp2 = 74u; }
    v = __fadd_rn(c32, c75);
    if (v < b) { b = v; bp = 32u; }
    v2 = __fadd_rn(c96, c11);
    if (v2 < b2) { b2 = v2; bp2 = 96u; }
    v = __fadd_rn(c34, c73);
    if (v < b) { b = v; bp = 34u; }
    v2 = __fadd_rn(c98, c9);
    if (v2 < b2) { b2 = v2; bp2 = 98u; }
    v = __fadd_rn(c40, c67);
    if (v < b) { b = v; bp = 40u; }
    v2 = __fadd_rn(c104, c3);
    if (v2 < b2) { b2 = v2; bp2 = 104u; }
    v = __fadd_rn(c42, c65);
    if (v < b) { b = v; bp = 42u; }
    v2 = __fadd_rn(c106, c1);
    if (v2 < b2) { b2 = v2; bp2 = 106u; }
    v = __fadd_rn(c64, c43);
    if (v < b) { b = v; bp = 64u; }
    if (b2 < b) { b = b2; bp = bp2; }
    c107 = __fadd_rn(b, A[107 * 32]);
    P[107 * 32] = (uint8_t)bp;
  }
  float c108;
  {
    float b = kTlInf, b2 = kTlInf, v, v2;
    uint32_t bp = 0xffu, bp2 = 0xffu;
    v = __fadd_rn(c8, c100);
    if (v < b) { b = v; bp = 8u; }
    v2 = __fadd_rn(c72, c36);
    if (v2 < b2) { b2 = v2; bp2 = 72u; }
    v = __fadd_rn(c32, c76);
    if (v < b) { b = v; bp = 32u; }
    v2 = __fadd_rn(c96, c12);
    if (v2 < b2) { b2 = v2; bp2 = 96u; }
    v = __fadd_rn(c40, c68);
    if (v < b) { b = v; bp = 40u; }
    v2 = __fadd_rn(c104, c4);
    if (v2 < b2) { b2 = v2; bp2 = 104u; }
    v = __fadd_rn(c64, c44);
    if (v < b) { b = v; bp = 64u; }
    if (b2 < b) { b = b2; bp = bp2; }
    c108 = __fadd_rn(b, A[108 * 32]);
    P[108 * 32] = (uint8_t)bp;
  }
  float c109;
  {
    float b = kTlInf, b2 = kTlInf, v, v2;
    uint32_t bp = 0xffu, bp2 = 0xffu;
    v = __fadd_rn(c4, c105);
    if (v < b) { b = v; bp = 4u; }
    v2 = __fadd_rn(c68, c41);
    if (v2 < b2) { b2 = v2; bp2 = 68u; }
    v = __fadd_rn(c8, c101);
    if (v < b) { b = v; bp = 8u; }
    v2 = __fadd_rn(c72, c37);
    if (v2 < b2) { b2 = v2; bp2 = 72u; }
    v = __fadd_rn(c12, c97);
    if (v < b) { b = v; bp = 12u; }
    v2 = __fadd_rn(c76, c33);
    if (v2 < b2) { b2 = v2; bp2 = 76u; }
    v = __fadd_rn(c32, c77);
    if (v < b) { b = v; bp = 32u; }
    v2 = __fadd_rn(c96, c13);
    if (v2 < b2) { b2 = v2; bp2 = 96u; }
    v = __fadd_rn(c36, c73);
    if (v < b) { b = v; bp = 36u; }
    v2 = __fadd_rn(c100, c9);
    if (v2 < b2) { b2 = v2; bp2 = 100u; }
    v = __fadd_rn(c40, c69);
    if (v < b) { b = v; bp = 40u; }
    v2 = __fadd_rn(c104, c5);
    if (v2 < b2) { b2 = v2; bp2 = 104u; }
    v = __fadd_rn(c44, c65);
    if (v < b) { b = v; bp = 44u; }
    v2 = __fadd_rn(c108, c1);
    if (v2 < b2) { b2 = v2; bp2 = 108u; }
    v = __fadd_rn(c64, c45);
    if (v < b) { b = v; bp = 64u; }
    if (b2 < b) { b = b2; bp = bp2; }
    c109 = __fadd_rn(b, A[109 * 32]);
    P[109 * 32] = (uint8_t)bp;
  }
  float c110;
  {
    float b = kTlInf, b2 = kTlInf, v, v2;
    uint32_t bp = 0xffu, bp2 = 0xffu;
    v = __fadd_rn(c4, c106);
    if (v < b) { b = v; bp = 4u; }
    v2 = __fadd_rn(c68, c42);
    if (v2 < b2) { b2 = v2; bp2 = 68u; }
    v = __fadd_rn(c8, c102);
    if (v < b) { b = v; bp = 8u; }
    v2 = __fadd_rn(c72, c38);
    if (v2 < b2) { b2 = v2; bp2 = 72u; }
    v = __fadd_rn(c12, c98);
    if (v < b) { b = v; bp = 12u; }
    v2 = __fadd_rn(c76, c34);
    if (v2 < b2) { b2 = v2; bp2 = 76u; }
    v = __fadd_rn(c32, c78);
    if (v < b) { b = v; bp = 32u; }
    v2 = __fadd_rn(c96, c14);
    if (v2 < b2) { b2 = v2; bp2 = 96u; }
    v = __fadd_rn(c36, c74);
    if (v < b) { b = v; bp = 36u; }
    v2 = __fadd_rn(c100, c10);
    if (v2 < b2) { b2 = v2; bp2 = 100u; }
    v = __fadd_rn(c40, c70);
    if (v < b) { b = v; bp = 40u; }
    v2 = __fadd_rn(c104, c6);
    if (v2 < b2) { b2 = v2; bp2 = 104u; }
    v = __fadd_rn(c44, c66);
    if (v < b) { b = v; bp = 44u; }
    v2 = __fadd_rn(c108, c2);
    if (v2 < b2) { b2 = v2; bp2 = 108u; }
    v = __fadd_rn(c64, c46);
    if (v < b) { b = v; bp = 64u; }
    if (b2 < b) { b = b2; bp = bp2; }
    c110 = __fadd_rn(b, A[110 * 32]);
    P[110 * 32] = (uint8_t)bp;
  }
  float c111;
  {
    float b = kTlInf, b2 = kTlInf, v, v2;
    uint32_t bp = 0xffu, bp2 = 0xffu;
    v = __fadd_rn(c2, c109);
    if (v < b) { b = v; bp = 2u; }
    v2 = __fadd_rn(c66, c45);
    if (v2 < b2) { b2 = v2; bp2 = 66u; }
    v = __fadd_rn(c4, c107);
    if (v < b) { b = v; bp = 4u; }
    v2 = __fadd_rn(c68, c43);
    if (v2 < b2) { b2 = v2; bp2 = 68u; }
    v = __fadd_rn(c6, c105);
    if (v < b) { b = v; bp = 6u; }
    v2 = __fadd_rn(c70, c41);
    if (v2 < b2) { b2 = v2; bp2 = 70u; }
    v = __fadd_rn(c8, c103);
    if (v < b) { b = v; bp = 8u; }
    v2 = __fadd_rn(c72, c39);
    if (v2 < b2) { b2 = v2; bp2 = 72u; }
    v = __fadd_rn(c10, c101);
    if (v < b) { b = v; bp = 10u; }
    v2 = __fadd_rn(c74, c37);
    if (v2 < b2) { b2 = v2; bp2 = 74u; }
    v = __fadd_rn(c12, c99);
    if (v < b) { b = v; bp = 12u; }
    v2 = __fadd_rn(c76, c35);
    if (v2 < b2) { b2 = v2; bp2 = 76u; }
    v = __fadd_rn(c14, c97);
    if (v < b) { b = v; bp = 14u; }
    v2 = __fadd_rn(c78, c33);
    if (v2 < b2) { b2 = v2; bp2 = 78u; }
    v = __fadd_rn(c32, c79);
    if (v < b) { b = v; bp = 32u; }
    v2 = __fadd_rn(c96, c15);
    if (v2 < b2) { b2 = v2; bp2 = 96u; }
    v = __fadd_rn(c34, c77);
    if (v < b) { b = v; bp = 34u; }
    v2 = __fadd_rn(c98, c13);
    if (v2 < b2) { b2 = v2; bp2 = 98u; }
    v = __fadd_rn(c36, c75);
    if (v < b) { b = v; bp = 36u; }
    v2 = __fadd_rn(c100, c11);
    if (v2 < b2) { b2 = v2; bp2 = 100u; }
    v = __fadd_rn(c38, c73);
    if (v < b) { b = v; bp = 38u; }
    v2 = __fadd_rn(c102, c9);
    if (v2 < b2) { b2 = v2; bp2 = 102u; }
    v = __fadd_rn(c40, c71);
    if (v < b) { b = v; bp = 40u; }
    v2 = __fadd_rn(c104, c7);
    if (v2 < b2) { b2 = v2; bp2 = 104u; }
    v = __fadd_rn(c42, c69);
    if (v < b) { b = v; bp = 42u; }
    v2 = __fadd_rn(c106, c5);
    if (v2 < b2) { b2 = v2; bp2 = 106u; }
    v = __fadd_rn(c44, c67);
    if (v < b) { b = v; bp = 44u; }
    v2 = __fadd_rn(c108, c3);
    if (v2 < b2) { b2 = v2; bp2 = 108u; }
    v = __fadd_rn(c46, c65);
    if (v < b) { b = v; bp = 46u; }
    v2 = __fadd_rn(c110, c1);
    if (v2 < b2) { b2 = v2; bp2 = 110u; }
    v = __fadd_rn(c64, c47);
    if (v < b) { b = v; bp = 64u; }
    if (b2 < b) { b = b2; bp = bp2; }
    c111 = __fadd_rn(b, A[111 * 32]);
    P[111 * 32] = (uint8_t)bp;
  }
  float c112;
  {
    float b = kTlInf, v;
    uint32_t bp = 0xffu;
    v = __fadd_rn(c32, c80);
    if (v < b) { b = v; bp = 32u; }
    v = __fadd_rn(c64, c48);
    if (v < b) { b = v; bp = 64u; }
    v = __fadd_rn(c96, c16);
    if (v < b) { b = v; bp = 96u; }
    c112 = __fadd_rn(b, A[112 * 32]);
    P[112 * 32] = (uint8_t)bp;
  }
  float c113;
  {
    float b = kTlInf, b2 = kTlInf, v, v2;
    uint32_t bp = 0xffu, bp2 = 0xffu;
    v = __fadd_rn(c16, c97);
    if (v < b) { b = v; bp = 16u; }
    v2 = __fadd_rn(c80, c33);
    if (v2 < b2) { b2 = v2; bp2 = 80u; }
    v = __fadd_rn(c32, c81);
    if (v < b) { b = v; bp = 32u; }
    v2 = __fadd_rn(c96, c17);
    if (v2 < b2) { b2 = v2; bp2 = 96u; }
    v = __fadd_rn(c48, c65);
    if (v < b) { b = v; bp = 48u; }
    v2 = __fadd_rn(c112, c1);
    if (v2 < b2) { b2 = v2; bp2 = 112u; }
    v = __fadd_rn(c64, c49);
    if (v < b) { b = v; bp = 64u; }
    if (b2 < b) { b = b2; bp = bp2; }
    c113 = __fadd_rn(b, A[113 * 32]);
    P[113 * 32] = (uint8_t)bp;
  }
  float c114;
  {
    float b = kTlInf, b2 = kTlInf, v, v2;
    uint32_t bp = 0xffu, bp2 = 0xffu;
    v = __fadd_rn(c16, c98);
    if (v < b) { b = v; bp = 16u; }
    v2 = __fadd_rn(c80, c34);
    if (v2 < b2) { b2 = v2; bp2 = 80u; }
    v = __fadd_rn(c32, c82);
    if (v < b) { b = v; bp = 32u; }
    v2 = __fadd_rn(c96, c18);
    if (v2 < b2) { b2 = v2; bp2 = 96u; }
    v = __fadd_rn(c48, c66);
    if (v < b) { b = v; bp = 48u; }
    v2 = __fadd_rn(c112, c2);
    if (v2 < b2) { b2 = v2; bp2 = 112u; }
    v = __fadd_rn(c64, c50);
    if (v < b) { b = v; bp = 64u; }
    if (b2 < b) { b = b2; bp = bp2; }
    c114 = __fadd_rn(b, A[114 * 32]);
    P[114 * 32] = (uint8_t)bp;
  }
  float c115;
  {
    float b = kTlInf, b2 = kTlInf, v, v2;
    uint32_t bp = 0xffu, bp2 = 0xffu;
    v = __fadd_rn(c2, c113);
    if (v < b) { b = v; bp = 2u; }
    v2 = __fadd_rn(c66, c49);
    if (v2 < b2) { b2 = v2; bp2 = 66u; }
    v = __fadd_rn(c16, c99);
    if (v < b) { b = v; bp = 16u; }
    v2 = __fadd_rn(c80, c35);
    if (v2 < b2) { b2 = v2; bp2 = 80u; }
    v = __fadd_rn(c18, c97);
    if (v < b) { b = v; bp = 18u; }
    v2 = __fadd_rn(c82, c33);
    if (v2 < b2) { b2 = v2; bp2 = 82u; }
    v = __fadd_rn(c32, c83);
    if (v < b) { b = v; bp = 32u; }
    v2 = __fadd_rn(c96, c19);
    if (v2 < b2) { b2 = v2; bp2 = 96u; }
    v = __fadd_rn(c34, c81);
    if (v < b) { b = v; bp = 34u; }
    v2 = __fadd_rn(c98, c17);
    if (v2 < b2) { b2 = v2; bp2 = 98u; }
    v = __fadd_rn(c48, c67);
    if (v < b) { b = v; bp = 48u; }
    v2 = __fadd_rn(c112, c3);
    if (v2 < b2) { b2 = v2; bp2 = 112u; }
    v = __fadd_rn(c50, c65);
    if (v < b) { b = v; bp = 50u; }
    v2 = __fadd_rn(c114, c1);
    if (v2 < b2) { b2 = v2; bp2 = 114u; }
    v = __fadd_rn(c64, c51);
    if (v < b) { b = v; bp = 64u; }
    if (b2 < b) { b = b2; bp = bp2; }
    c115 = __fadd_rn(b, A[115 * 32]);
    P[115 * 32] = (uint8_t)bp;
  }
  float c116;
  {
    float b = kTlInf, b2 = kTlInf, v, v2;
    uint32_t bp = 0xffu, bp2 = 0xffu;
    v = __fadd_rn(c16, c100);
    if (v < b) { b = v; bp = 16u; }
    v2 = __fadd_rn(c80, c36);
    if (v2 < b2) { b2 = v2; bp2 = 80u; }
    v = __fadd_rn(c32, c84);
    if (v < b) { b = v; bp = 32u; }
    v2 = __fadd_rn(c96, c20);
    if (v2 < b2) { b2 = v2; bp2 = 96u; }
    v = __fadd_rn(c48, c68);
    if (v < b) { b = v; bp = 48u; }
    v2 = __fadd_rn(c112, c4);
    if (v2 < b2) { b2 = v2; bp2 = 112u; }
    v = __fadd_rn(c64, c52);
    if (v < b) { b = v; bp = 64u; }
    if (b2 < b) { b = b2; bp = bp2; }
    c116 = __fadd_rn(b, A[116 * 32]);
    P[116 * 32] = (uint8_t)bp;
  }
  float c117;
  {
    float b = kTlInf, b2 = kTlInf, v, v2;
    uint32_t bp = 0xffu, bp2 = 0xffu;
    v = __fadd_rn(c4, c113);
    if (v < b) { b = v; bp = 4u; }
    v2 = __fadd_rn(c68, c49);
    if (v2 < b2) { b2 = v2; bp2 = 68u; }
    v = __fadd_rn(c16, c101);
    if (v < b) { b = v; bp = 16u; }
    v2 = __fadd_rn(c80, c37);
    if (v2 < b2) { b2 = v2; bp2 = 80u; }
    v = __fadd_rn(c20, c97);
    if (v < b) { b = v; bp = 20u; }
    v2 = __fadd_rn(c84, c33);
    if (v2 < b2) { b2 = v2; bp2 = 84u; }
    v = __fadd_rn(c32, c85);
    if (v < b) { b = v; bp = 32u; }
    v2 = __fadd_rn(c96, c21);
    if (v2 < b2) { b2 = v2; bp2 = 96u; }
    v = __fadd_rn(c36, c81);
    if (v < b) { b = v; bp = 36u; }
    v2 = __fadd_rn(c100, c17);
    if (v2 < b2) { b2 = v2; bp2 = 100u; }
    v = __fadd_rn(c48, c69);
    if (v < b) { b = v; bp = 48u; }
    v2 = __fadd_rn(c112, c5);
    if (v2 < b2) { b2 = v2; bp2 = 112u; }
    v = __fadd_rn(c52, c65);
    if (v < b) { b = v; bp = 52u; }
    v2 = __fadd_rn(c116, c1);
    if (v2 < b2) { b2 = v2; bp2 = 116u; }
    v = __fadd_rn(c64, c53);
    if (v < b) { b = v; bp = 64u; }
    if (b2 < b) { b = b2; bp = bp2; }
    c117 = __fadd_rn(b, A[117 * 32]);
    P[117 * 32] = (uint8_t)bp;
  }
  float c118;
  {
    float b = kTlInf, b2 = kTlInf, v, v2;
    uint32_t bp = 0xffu, bp2 = 0xffu;
    v = __fadd_rn(c4, c114);
    if (v < b) { b = v; bp = 4u; }
    v2 = __fadd_rn(c68, c50);
    if (v2 < b2) { b2 = v2; bp2 = 68u; }
    v = __fadd_rn(c16, c102);
    if (v < b) { b = v; bp = 16u; }
    v2 = __fadd_rn(c80, c38);
    if (v2 < b2) { b2 = v2; bp2 = 80u; }
    v = __fadd_rn(c20, c98);
    if (v < b) { b = v; bp = 20u; }
    v2 = __fadd_rn(c84, c34);
    if (v2 < b2) { b2 = v2; bp2 = 84u; }
    v = __fadd_rn(c32, c86);
    if (v < b) { b = v; bp = 32u; }
    v2 = __fadd_rn(c96, c22);
    if (v2 < b2) { b2 = v2; bp2 = 96u; }
    v = __fadd_rn(c36, c82);
    if (v < b) { b = v; bp = 36u; }
    v2 = __fadd_rn(c100, c18);
    if (v2 < b2) { b2 = v2; bp2 = 100u; }
    v = __fadd_rn(c48, c70);
    if (v < b) { b = v; bp = 48u; }
    v2 = __fadd_rn(c112, c6);
    if (v2 < b2) { b2 = v2; bp2 = 112u; }
    v = __fadd_rn(c52, c66);
    if (v < b) { b = v; bp = 52u; }
    v2 = __fadd_rn(c116, c2);
    if (v2 < b2) { b2 = v2; bp2 = 116u; }
    v = __fadd_rn(c64, c54);
    if (v < b) { b = v; bp = 64u; }
    if (b2 < b) { b = b2; bp = bp2; }
    c118 = __fadd_rn(b, A[118 * 32]);
    P[118 * 32] = (uint8_t)bp;
  }
  float c119;
  {
    float b = kTlInf, b2 = kTlInf, v, v2;
    uint32_t bp = 0xffu, bp2 = 0xffu;
    v = __fadd_rn(c2, c117);
    if (v < b) { b = v; bp = 2u; }
    v2 = __fadd_rn(c66, c53);
    if (v2 < b2) { b2 = v2; bp2 = 66u; }
    v = __fadd_rn(c4, c115);
    if (v < b) { b = v; bp = 4u; }
    v2 = __fadd_rn(c68, c51);
    if (v2 < b2) { b2 = v2; bp2 = 68u; }
    v = __fadd_rn(c6, c113);
    if (v < b) { b = v; bp = 6u; }
    v2 = __fadd_rn(c70, c49);
    if (v2 < b2) { b2 = v2; bp2 = 70u; }
    v = __fadd_rn(c16, c103);
    if (v < b) { b = v; bp = 16u; }
    v2 = __fadd_rn(c80, c39);
    if (v2 < b2) { b2 = v2; bp2 = 80u; }
    v = __fadd_rn(c18, c101);
    if (v < b) { b = v; bp = 18u; }
    v2 = __fadd_rn(c82, c37);
    if (v2 < b2) { b2 = v2; bp2 = 82u; }
    v = __fadd_rn(c20, c99);
    if (v < b) { b = v; bp = 20u; }
    v2 = __fadd_rn(c84, c35);
    if (v2 < b2) { b2 = v2; bp2 = 84u; }
    v = __fadd_rn(c22, c97);
    if (v < b) { b = v; bp = 22u; }
    v2 = __fadd_rn(c86, c33);
    if (v2 < b2) { b2 = v2; bp2 = 86u; }
    v = __fadd_rn(c32, c87);
    if (v < b) { b = v; bp = 32u; }
    v2 = __fadd_rn(c96, c23);
    if (v2 < b2) { b2 = v2; bp2 = 96u; }
    v = __fadd_rn(c34, c85);
    if (v < b) { b = v; bp = 34u; }
    v2 = __fadd_rn(c98, c21);
    if (v2 < b2) { b2 = v2; bp2 = 98u; }
    v = __fadd_rn(c36, c83);
    if (v < b) { b = v; bp = 36u; }
    v2 = __fadd_rn(c100, c19);
    if (v2 < b2) { b2 = v2; bp2 = 100u; }
    v = __fadd_rn(c38, c81);
    if (v < b) { b = v; bp = 38u; }
    v2 = __fadd_rn(c102, c17);
    if (v2 < b2) { b2 = v2; bp2 = 102u; }
    v = __fadd_rn(c48, c71);
    if (v < b) { b = v; bp = 48u; }
    v2 = __fadd_rn(c112, c7);
    if (v2 < b2) { b2 = v2; bp2 = 112u; }
    v = __fadd_rn(c50, c69);
    if (v < b) { b = v; bp = 50u; }
    v2 = __fadd_rn(c114, c5);
    if (v2 < b2) { b2 = v2; bp2 = 114u; }
    v = __fadd_rn(c52, c67);
    if (v < b) { b = v; bp = 52u; }
    v2 = __fadd_rn(c116, c3);
    if (v2 < b2) { b2 = v2; bp2 = 116u; }
    v = __fadd_rn(c54, c65);
    if (v < b) { b = v; bp = 54u; }
    v2 = __fadd_rn(c118, c1);
    if (v2 < b2) { b2 = v2; bp2 = 118u; }
    v = __fadd_rn(c64, c55);
    if (v < b) { b = v; bp = 64u; }
    if (b2 < b) { b = b2; bp = bp2; }
    c119 = __fadd_rn(b, A[119 * 32]);
    P[119 * 32] = (uint8_t)bp;
  }
  float c120;
  {
    float b = kTlInf, b2 = kTlInf, v, v2;
    uint32_t bp = 0xffu, bp2 = 0xffu;
    v = __fadd_rn(c16, c104);
    if (v < b) { b = v; bp = 16u; }
    v2 = __fadd_rn(c80, c40);
    if (v2 < b2) { b2 = v2; bp2 = 80u; }
    v = __fadd_rn(c32, c88);
    if (v < b) { b = v; bp = 32u; }
    v2 = __fadd_rn(c96, c24);
    if (v2 < b2) { b2 = v2; bp2 = 96u; }
    v = __fadd_rn(c48, c72);
    if (v < b) { b = v; bp = 48u; }
    v2 = __fadd_rn(c112, c8);
    if (v2 < b2) { b2 = v2; bp2 = 112u; }
    v = __fadd_rn(c64, c56);
    if (v < b) { b = v; bp = 64u; }
    if (b2 < b) { b = b2; bp = bp2; }
    c120 = __fadd_rn(b, A[120 * 32]);
    P[120 * 32] = (uint8_t)bp;
  }
  float c121;
  {
    float b = kTlInf, b2 = kTlInf, v, v2;
    uint32_t bp = 0xffu, bp2 = 0xffu;
    v = __fadd_rn(c8, c113);
    if (v < b) { b = v; bp = 8u; }
    v2 = __fadd_rn(c72, c49);
    if (v2 < b2) { b2 = v2; bp2 = 72u; }
    v = __fadd_rn(c16, c105);
    if (v < b) { b = v; bp = 16u; }
    v2 = __fadd_rn(c80, c41);
    if (v2 < b2) { b2 = v2; bp2 = 80u; }
    v = __fadd_rn(c24, c97);
    if (v < b) { b = v; bp = 24u; }
    v2 = __fadd_rn(c88, c33);
    if (v2 < b2) { b2 = v2; bp2 = 88u; }
    v = __fadd_rn(c32, c89);
    if (v < b) { b = v; bp = 32u; }
    v2 = __fadd_rn(c96, c25);
    if (v2 < b2) { b2 = v2; bp2 = 96u; }
    v = __fadd_rn(c40, c81);
    if (v < b) { b = v; bp = 40u; }
    v2 = __fadd_rn(c104, c17);
    if (v2 < b2) { b2 = v2; bp2 = 104u; }
    v = __fadd_rn(c48, c73);
    if (v < b) { b = v; bp = 48u; }
    v2 = __fadd_rn(c112, c9);
    if (v2 < b2) { b2 = v2; bp2 = 112u; }
    v = __fadd_rn(c56, c65);
    if (v < b) { b = v; bp = 56u; }
    v2 = __fadd_rn(c120, c1);
    if (v2 < b2) { b2 = v2; bp2 = 120u; }
    v = __fadd_rn(c64, c57);
    if (v < b) { b = v; bp = 64u; }
    if (b2 < b) { b = b2; bp = bp2; }
    c121 = __fadd_rn(b, A[121 * 32]);
    P[121 * 32] = (uint8_t)bp;
  }
  float c122;
  {
    float b = kTlInf, b2 = kTlInf, v, v2;
    uint32_t bp = 0xffu, bp2 = 0xffu;
    v = __fadd_rn(c8, c114);
    if (v < b) { b = v; bp = 8u; }
    v2 = __fadd_rn(c72, c50);
    if (v2 < b2) { b2 = v2; bp2 = 72u; }
    v = __fadd_rn(c16, c106);
    if (v < b) { b = v; bp = 16u; }
    v2 = __fadd_rn(c80, c42);
    if (v2 < b2) { b2 = v2; bp2 = 80u; }
    v = __fadd_rn(c24, c98);
    if (v < b) { b = v; bp = 24u; }
    v2 = __fadd_rn(c88, c34);
    if (v2 < b2) { b2 = v2; bp2 = 88u; }
    v = __fadd_rn(c32, c90);
    if (v < b) { b = v; bp = 32u; }
    v2 = __fadd_rn(c96, c26);
    if (v2 < b2) { b2 = v2; bp2 = 96u; }
    v = __fadd_rn(c40, c82);
    if (v < b) { b = v; bp = 40u; }
    v2 = __fadd_rn(c104, c18);
    if (v2 < b2) { b2 = v2; bp2 = 104u; }
    v = __fadd_rn(c48, c74);
    if (v < b) { b = v; bp = 48u; }
    v2 = __fadd_rn(c112, c10);
    if (v2 < b2) { b2 = v2; bp2 = 112u; }
    v = __fadd_rn(c56, c66);
    if (v < b) { b = v; bp = 56u; }
    v2 = __fadd_rn(c120, c2);
    if (v2 < b2) { b2 = v2; bp2 = 120u; }
    v = __fadd_rn(c64, c58);
    if (v < b) { b = v; bp = 64u; }
    if (b2 < b) { b = b2; bp = bp2; }
    c122 = __fadd_rn(b, A[122 * 32]);
    P[122 * 32] = (uint8_t)bp;
  }
  float c123;
  {
    float b = kTlInf, b2 = kTlInf, v, v2;
    uint32_t bp = 0xffu, bp2 = 0xffu;
    v = __fadd_rn(c2, c121);
    if (v < b) { b = v; bp = 2u; }
    v2 = __fadd_rn(c66, c57);
    if (v2 < b2) { b2 = v2; bp2 = 66u; }
    v = __fadd_rn(c8, c115);
    if (v < b) { b = v; bp = 8u; }
    v2 = __fadd_rn(c72, c51);
    if (v2 < b2) { b2 = v2; bp2 = 72u; }
    v = __fadd_rn(c10, c113);
    if (v < b) { b = v; bp = 10u; }
    v2 = __fadd_rn(c74, c49);
    if (v2 < b2) { b2 = v2; bp2 = 74u; }
    v = __fadd_rn(c16, c107);
    if (v < b) { b = v; bp = 16u; }
    v2 = __fadd_rn(c80, c43);
    if (v2 < b2) { b2 = v2; bp2 = 80u; }
    v = __fadd_rn(c18, c105);
    if (v < b) { b = v; bp = 18u; }
    v2 = __fadd_rn(c82, c41);
    if (v2 < b2) { b2 = v2; bp2 = 82u; }
    v = __fadd_rn(c24, c99);
    if (v < b) { b = v; bp = 24u; }
    v2 = __fadd_rn(c88, c35);
    if (v2 < b2) { b2 = v2; bp2 = 88u; }
    v = __fadd_rn(c26, c97);
    if (v < b) { b = v; bp = 26u; }
    v2 = __fadd_rn(c90, c33);
    if (v2 < b2) { b2 = v2; bp2 = 90u; }
    v = __fadd_rn(c32, c91);
    if (v < b) { b = v; bp = 32u; }
    v2 = __fadd_rn(c96, c27);
    if (v2 < b2) { b2 = v2; bp2 = 96u; }
    v = __fadd_rn(c34, c89);
    if (v < b) { b = v; bp = 34u; }
    v2 = __fadd_rn(c98, c25);
    if (v2 < b2) { b2 = v2; bp2 = 98u; }
    v = __fadd_rn(c40, c83);
    if (v < b) { b = v; bp = 40u; }
    v2 = __fadd_rn(c104, c19);
    if (v2 < b2) { b2 = v2; bp2 = 104u; }
    v = __fadd_rn(c42, c81);
    if (v < b) { b = v; bp = 42u; }
    v2 = __fadd_rn(c106, c17);
    if (v2 < b2) { b2 = v2; bp2 = 106u; }
    v = __fadd_rn(c48, c75);
    if (v < b) { b = v; bp = 48u; }
    v2 = __fadd_rn(c112, c11);
    if (v2 < b2) { b2 = v2; bp2 = 112u; }
    v = __fadd_rn(c50, c73);
    if (v < b) { b = v; bp = 50u; }
    v2 = __fadd_rn(c114, c9);
    if (v2 < b2) { b2 = v2; bp2 = 114u; }
    v = __fadd_rn(c56, c67);
    if (v < b) { b = v; bp = 56u; }
    v2 = __fadd_rn(c120, c3);
    if (v2 < b2) { b2 = v2; bp2 = 120u; }
    v = __fadd_rn(c58, c65);
    if (v < b) { b = v; bp = 58u; }
    v2 = __fadd_rn(c122, c1);
    if (v2 < b2) { b2 = v2; bp2 = 122u; }
    v = __fadd_rn(c64, c59);
    if (v < b) { b = v; bp = 64u; }
    if (b2 < b) { b = b2; bp = bp2; }
    c123 = __fadd_rn(b, A[123 * 32]);
    P[123 * 32] = (uint8_t)bp;
  }
  float c124;
  {
    float b = kTlInf, b2 = kTlInf, v, v2;
    uint32_t bp = 0xffu, bp2 = 0xffu;
    v = __fadd_rn(c8, c116);
    if (v < b) { b = v; bp = 8u; }
    v2 = __fadd_rn(c72, c52);
    if (v2 < b2) { b2 = v2; bp2 = 72u; }
    v = __fadd_rn(c16, c108);
    if (v < b) { b = v; bp = 16u; }
    v2 = __fadd_rn(c80, c44);
    if (v2 < b2) { b2 = v2; bp2 = 80u; }
    v = __fadd_rn(c24, c100);
    if (v < b) { b = v; bp = 24u; }
    v2 = __fadd_rn(c88, c36);
    if (v2 < b2) { b2 = v2; bp2 = 88u; }
    v = __fadd_rn(c32, c92);
    if (v < b) { b = v; bp = 32u; }
    v2 = __fadd_rn(c96, c28);
    if (v2 < b2) { b2 = v2; bp2 = 96u; }
    v = __fadd_rn(c40, c84);
    if (v < b) { b = v; bp = 40u; }
    v2 = __fadd_rn(c104, c20);
    if (v2 < b2) { b2 = v2; bp2 = 104u; }
    v = __fadd_rn(c48, c76);
    if (v < b) { b = v; bp = 48u; }
    v2 = __fadd_rn(c112, c12);
    if (v2 < b2) { b2 = v2; bp2 = 112u; }
    v = __fadd_rn(c56, c68);
    if (v < b) { b = v; bp = 56u; }
    v2 = __fadd_rn(c120, c4);
    if (v2 < b2) { b2 = v2; bp2 = 120u; }
    v = __fadd_rn(c64, c60);
    if (v < b) { b = v; bp = 64u; }
    if (b2 < b) { b = b2; bp = bp2; }
    c124 = __fadd_rn(b, A[124 * 32]);
    P[124 * 32] = (uint8_t)bp;
  }
  float c125;
  {
    float b = kTlInf, b2 = kTlInf, v, v2;
    uint32_t bp = 0xffu, bp2 = 0xffu;
    v = __fadd_rn(c4, c121);
    if (v < b) { b = v; bp = 4u; }
    v2 = __fadd_rn(c68, c57);
    if (v2 < b2) { b2 = v2; bp2 = 68u; }
    v = __fadd_rn(c8, c117);
    if (v < b) { b = v; bp = 8u; }
    v2 = __fadd_rn(c72, c53);
    if (v2 < b2) { b2 = v2; bp2 = 72u; }
    v = __fadd_rn(c12, c113);
    if (v < b) { b = v; bp = 12u; }
    v2 = __fadd_rn(c76, c49);
    if (v2 < b2) { b2 = v2; bp2 = 76u; }
    v = __fadd_rn(c16, c109);
    if (v < b) { b = v; bp = 16u; }
    v2 = __fadd_rn(c80, c45);
    if (v2 < b2) { b2 = v2; bp2 = 80u; }
    v = __fadd_rn(c20, c105);
    if (v < b) { b = v; bp = 20u; }
    v2 = __fadd_rn(c84, c41);
    if (v2 < b2) { b2 = v2; bp2 = 84u; }
    v = __fadd_rn(c24, c101);
    if (v < b) { b = v; bp = 24u; }
    v2 = __fadd_rn(c88, c37);
    if (v2 < b2) { b2 = v2; bp2 = 88u; }
    v = __fadd_rn(c28, c97);
    if (v < b) { b = v; bp = 28u; }
    v2 = __fadd_rn(c92, c33);
    if (v2 < b2) { b2 = v2; bp2 = 92u; }
    v = __fadd_rn(c32, c93);
    if (v < b) { b = v; bp = 32u; }
    v2 = __fadd_rn(c96, c29);
    if (v2 < b2) { b2 = v2; bp2 = 96u; }
    v = __fadd_rn(c36, c89);
    if (v < b) { b = v; bp = 36u; }
    v2 = __fadd_rn(c100, c25);
    if (v2 < b2) { b2 = v2; bp2 = 100u; }
    v = __fadd_rn(c40, c85);
    if (v < b) { b = v; bp = 40u; }
    v2 = __fadd_rn(c104, c21);
    if (v2 < b2) { b2 = v2; bp2 = 104u; }
    v = __fadd_rn(c44, c81);
    if (v < b) { b = v; bp = 44u; }
    v2 = __fadd_rn(c108, c17);
    if (v2 < b2) { b2 = v2; bp2 = 108u; }
    v = __fadd_rn(c48, c77);
    if (v < b) { b = v; bp = 48u; }
    v2 = __fadd_rn(c112, c13);
    if (v2 < b2) { b2 = v2; bp2 = 112u; }
    v = __fadd_rn(c52, c73);
    if (v < b) { b = v; bp = 52u; }
    v2 = __fadd_rn(c116, c9);
    if (v2 < b2) { b2 = v2; bp2 = 116u; }
    v = __fadd_rn(c56, c69);
    if (v < b) { b = v; bp = 56u; }
    v2 = __fadd_rn(c120, c5);
    if (v2 < b2) { b2 = v2; bp2 = 120u; }
    v = __fadd_rn(c60, c65);
    if (v < b) { b = v; bp = 60u; }
    v2 = __fadd_rn(c124, c1);
    if (v2 < b2) { b2 = v2; bp2 = 124u; }
    v = __fadd_rn(c64, c61);
    if (v < b) { b = v; bp = 64u; }
    if (b2 < b) { b = b2; bp = bp2; }
    c125 = __fadd_rn(b, A[125 * 32]);
    P[125 * 32] = (uint8_t)bp;
  }
  float c126;
  {
    float b = kTlInf, b2 = kTlInf, v, v2;
    uint32_t bp = 0xffu, bp2 = 0xffu;
    v = __fadd_rn(c4, c122);
    if (v < b) { b = v; bp = 4u; }
    v2 = __fadd_rn(c68, c58);
    if (v2 < b2) { b2 = v2; bp2 = 68u; }
    v = __fadd_rn(c8, c118);
    if (v < b) { b = v; bp = 8u; }
    v2 = __fadd_rn(c72, c54);
    if (v2 < b2) { b2 = v2; bp2 = 72u; }
    v = __fadd_rn(c12, c114);
    if (v < b) { b = v; bp = 12u; }
    v2 = __fadd_rn(c76, c50);
    if (v2 < b2) { b2 = v2; bp2 = 76u; }
    v = __fadd_rn(c16, c110);
    if (v < b) { b = v; bp = 16u; }
    v2 = __fadd_rn(c80, c46);
    if (v2 < b2) { b2 = v2; bp2 = 80u; }
    v = __fadd_rn(c20, c106);
    if (v < b) { b = v; bp = 20u; }
    v2 = __fadd_rn(c84, c42);
    if (v2 < b2) { b2 = v2; bp2 = 84u; }
    v = __fadd_rn(c24, c102);
    if (v < b) { b = v; bp = 24u; }
    v2 = __fadd_rn(c88, c38);
    if (v2 < b2) { b2 = v2; bp2 = 88u; }
    v = __fadd_rn(c28, c98);
    if (v < b) { b = v; bp = 28u; }
    v2 = __fadd_rn(c92, c34);
    if (v2 < b2) { b2 = v2; bp2 = 92u; }
    v = __fadd_rn(c32, c94);
    if (v < b) { b = v; bp = 32u; }
    v2 = __fadd_rn(c96, c30);
    if (v2 < b2) { b2 = v2; bp2 = 96u; }
    v = __fadd_rn(c36, c90);
    if (v < b) { b = v; bp = 36u; }
    v2 = __fadd_rn(c100, c26);
    if (v2 < b2) { b2 = v2; bp2 = 100u; }
    v = __fadd_rn(c40, c86);
    if (v < b) { b = v; bp = 40u; }
    v2 = __fadd_rn(c104, c22);
    if (v2 < b2) { b2 = v2; bp2 = 104u; }
    v = __fadd_rn(c44, c82);
    if (v < b) { b = v; bp = 44u; }
    v2 = __fadd_rn(c108, c18);
    if (v2 < b2) { b2 = v2; bp2 = 108u; }
    v = __fadd_rn(c48, c78);
    if (v < b) { b = v; bp = 48u; }
    v2 = __fadd_rn(c112, c14);
    if (v2 < b2) { b2 = v2; bp2 = 112u; }
    v = __fadd_rn(c52, c74);
    if (v < b) { b = v; bp = 52u; }
    v2 = __fadd_rn(c116, c10);
    if (v2 < b2) { b2 = v2; bp2 = 116u; }
    v = __fadd_rn(c56, c70);
    if (v < b) { b = v; bp = 56u; }
    v2 = __fadd_rn(c120, c6);
    if (v2 < b2) { b2 = v2; bp2 = 120u; }
    v = __fadd_rn(c60, c66);
    if (v < b) { b = v; bp = 60u; }
    v2 = __fadd_rn(c124, c2);
    if (v2 < b2) { b2 = v2; bp2 = 124u; }
    v = __fadd_rn(c64, c62);
    if (v < b) { b = v; bp = 64u; }
    if (b2 < b) { b = b2; bp = bp2; }
    c126 = __fadd_rn(b, A[126 * 32]);
    P[126 * 32] = (uint8_t)bp;
  }
  {
    float b = kTlInf, b2 = kTlInf, v, v2;
    uint32_t bp = 0xffu, bp2 = 0xffu;
    v = __fadd_rn(c2, c125);
    if (v < b) { b = v; bp = 2u; }
    v2 = __fadd_rn(c66, c61);
    if (v2 < b2) { b2 = v2; bp2 = 66u; }
    v = __fadd_rn(c4, c123);
    if (v < b) { b = v; bp = 4u; }
    v2 = __fadd_rn(c68, c59);
    if (v2 < b2) { b2 = v2; bp2 = 68u; }
    v = __fadd_rn(c6, c121);
    if (v < b) { b = v; bp = 6u; }
    v2 = __fadd_rn(c70, c57);
    if (v2 < b2) { b2 = v2; bp2 = 70u; }
    v = __fadd_rn(c8, c119);
    if (v < b) { b = v; bp = 8u; }
    v2 = __fadd_rn(c72, c55);
    if (v2 < b2) { b2 = v2; bp2 = 72u; }
    v = __fadd_rn(c10, c117);
    if (v < b) { b = v; bp = 10u; }
    v2 = __fadd_rn(c74, c53);
    if (v2 < b2) { b2 = v2; bp2 = 74u; }
    v = __fadd_rn(c12, c115);
    if (v < b) { b = v; bp = 12u; }
    v2 = __fadd_rn(c76, c51);
    if (v2 < b2) { b2 = v2; bp2 = 76u; }
    v = __fadd_rn(c14, c113);
    if (v < b) { b = v; bp = 14u; }
    v2 = __fadd_rn(c78, c49);
    if (v2 < b2) { b2 = v2; bp2 = 78u; }
    v = __fadd_rn(c16, c111);
    if (v < b) { b = v; bp = 16u; }
    v2 = __fadd_rn(c80, c47);
    if (v2 < b2) { b2 = v2; bp2 = 80u; }
    v = __fadd_rn(c18, c109);
    if (v < b) { b = v; bp = 18u; }
    v2 = __fadd_rn(c82, c45);
    if (v2 < b2) { b2 = v2; bp2 = 82u; }
    v = __fadd_rn(c20, c107);
    if (v < b) { b = v; bp = 20u; }
    v2 = __fadd_rn(c84, c43);
    if (v2 < b2) { b2 = v2; bp2 = 84u; }
    v = __fadd_rn(c22, c105);
    if (v < b) { b = v; bp = 22u; }
    v2 = __fadd_rn(c86, c41);
    if (v2 < b2) { b2 = v2; bp2 = 86u; }
    v = __fadd_rn(c24, c103);
    if (v < b) { b = v; bp = 24u; }
    v2 = __fadd_rn(c88, c39);
    if (v2 < b2) { b2 = v2; bp2 = 88u; }
    v = __fadd_rn(c26, c101);
    if (v < b) { b = v; bp = 26u; }
    v2 = __fadd_rn(c90, c37);
    if (v2 < b2) { b2 = v2; bp2 = 90u; }
    v = __fadd_rn(c28, c99);
    if (v < b) { b = v; bp = 28u; }
    v2 = __fadd_rn(c92, c35);
    if (v2 < b2) { b2 = v2; bp2 = 92u; }
    v = __fadd_rn(c30, c97);
    if (v < b) { b = v; bp = 30u; }
    v2 = __fadd_rn(c94, c33);
    if (v2 < b2) { b2 = v2; bp2 = 94u; }
    v = __fadd_rn(c32, c95);
    if (v < b) { b = v; bp = 32u; }
    v2 = __fadd_rn(c96, c31);
    if (v2 < b2) { b2 = v2; bp2 = 96u; }
    v = __fadd_rn(c34, c93);
    if (v < b) { b = v; bp = 34u; }
    v2 = __fadd_rn(c98, c29);
    if (v2 < b2) { b2 = v2; bp2 = 98u; }
    v = __fadd_rn(c36, c91);
    if (v < b) { b = v; bp = 36u; }
    v2 = __fadd_rn(c100, c27);
    if (v2 < b2) { b2 = v2; bp2 = 100u; }
    v = __fadd_rn(c38, c89);
    if (v < b) { b = v; bp = 38u; }
    v2 = __fadd_rn(c102, c25);
    if (v2 < b2) { b2 = v2; bp2 = 102u; }
    v = __fadd_rn(c40, c87);
    if (v < b) { b = v; bp = 40u; }
    v2 = __fadd_rn(c104, c23);
    if (v2 < b2) { b2 = v2; bp2 = 104u; }
    v = __fadd_rn(c42, c85);
    if (v < b) { b = v; bp = 42u; }
    v2 = __fadd_rn(c106, c21);
    if (v2 < b2) { b2 = v2; bp2 = 106u; }
    v = __fadd_rn(c44, c83);
    if (v < b) { b = v; bp = 44u; }
    v2 = __fadd_rn(c108, c19);
    if (v2 < b2) { b2 = v2; bp2 = 108u; }
    v = __fadd_rn(c46, c81);
    if (v < b) { b = v; bp = 46u; }
    v2 = __fadd_rn(c110, c17);
    if (v2 < b2) { b2 = v2; bp2 = 110u; }
    v = __fadd_rn(c48, c79);
    if (v < b) { b = v; bp = 48u; }
    v2 = __fadd_rn(c112, c15);
    if (v2 < b2) { b2 = v2; bp2 = 112u; }
    v = __fadd_rn(c50, c77);
    if (v < b) { b = v; bp = 50u; }
    v2 = __fadd_rn(c114, c13);
    if (v2 < b2) { b2 = v2; bp2 = 114u; }
    v = __fadd_rn(c52, c75);
    if (v < b) { b = v; bp = 52u; }
    v2 = __fadd_rn(c116, c11);
    if (v2 < b2) { b2 = v2; bp2 = 116u; }
    v = __fadd_rn(c54, c73);
    if (v < b) { b = v; bp = 54u; }
    v2 = __fadd_rn(c118, c9);
    if (v2 < b2) { b2 = v2; bp2 = 118u; }
    v = __fadd_rn(c56, c71);
    if (v < b) { b = v; bp = 56u; }
    v2 = __fadd_rn(c120, c7);
    if (v2 < b2) { b2 = v2; bp2 = 120u; }
    v = __fadd_rn(c58, c69);
    if (v < b) { b = v; bp = 58u; }
    v2 = __fadd_rn(c122, c5);
    if (v2 < b2) { b2 = v2; bp2 = 122u; }
    v = __fadd_rn(c60, c67);
    if (v < b) { b = v; bp = 60u; }
    v2 = __fadd_rn(c124, c3);
    if (v2 < b2) { b2 = v2; bp2 = 124u; }
    v = __fadd_rn(c62, c65);
    if (v < b) { b = v; bp = 62u; }
    v2 = __fadd_rn(c126, c1);
    if (v2 < b2) { b2 = v2; bp2 = 126u; }
    v = __fadd_rn(c64, c63);
    if (v < b) { b = v; bp = 64u; }
    if (b2 < b) { b = b2; bp = bp2; }
    P[127 * 32] = (uint8_t)bp;
  }
}

}  // namespace bvhgb
