// rb_common.cuh - pieces shared by the row-block Chebyshev steps (rb_spmm.cu,
// rbw_spmm.cu): the row-block geometry, the lane's 4 x 4 panel accumulator and
// the load forms. Included by .cu files only, inside their anonymous namespace.
#pragma once

constexpr int kRbRows = 4;          // rows per row block
constexpr int kRbSlotBytes = 20;    // 4 (column or window position) + 4 x 4 (values)

__device__ __forceinline__ unsigned long long pack2(float lo, float hi) {
  unsigned long long r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
  return r;
}
__device__ __forceinline__ float2 unpack2(unsigned long long r) {
  float2 f;
  asm("mov.b64 {%0, %1}, %2;" : "=f"(f.x), "=f"(f.y) : "l"(r));
  return f;
}
// acc += a * b on two FP32 lanes at once
__device__ __forceinline__ void fma2(unsigned long long& acc, unsigned long long a, unsigned long long b) {
  asm("fma.rn.f32x2 %0, %1, %2, %0;" : "+l"(acc) : "l"(a), "l"(b));
}

// A lane's share of one slot: rows 0..3 of the block += v[r] * x over its 4 columns.
template <bool PACKED>
struct PanelAcc;
template <>
struct PanelAcc<false> {
  float a[4][4];
  __device__ __forceinline__ void zero() {
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
      for (int c = 0; c < 4; ++c) a[r][c] = 0.f;
  }
  __device__ __forceinline__ void add(const float4& x, const float4& v) {
    const float w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      a[r][0] += w[r] * x.x;
      a[r][1] += w[r] * x.y;
      a[r][2] += w[r] * x.z;
      a[r][3] += w[r] * x.w;
    }
  }
  __device__ __forceinline__ void get(float (&o)[4][4]) const {
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
      for (int c = 0; c < 4; ++c) o[r][c] = a[r][c];
  }
};
// Pairs of rows (0,1), (2,3) per column: the value pairs come straight from the
// 16-byte load, each column of x is duplicated once per slot.
template <>
struct PanelAcc<true> {
  unsigned long long a[2][4];
  __device__ __forceinline__ void zero() {
#pragma unroll
    for (int p = 0; p < 2; ++p)
#pragma unroll
      for (int c = 0; c < 4; ++c) a[p][c] = 0ull;
  }
  __device__ __forceinline__ void add(const float4& x, const float4& v) {
    const unsigned long long v01 = pack2(v.x, v.y), v23 = pack2(v.z, v.w);
    const float xs[4] = {x.x, x.y, x.z, x.w};
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      const unsigned long long xx = pack2(xs[c], xs[c]);
      fma2(a[0][c], v01, xx);
      fma2(a[1][c], v23, xx);
    }
  }
  __device__ __forceinline__ void get(float (&o)[4][4]) const {
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      const float2 l = unpack2(a[0][c]), h = unpack2(a[1][c]);
      o[0][c] = l.x; o[1][c] = l.y; o[2][c] = h.x; o[3][c] = h.y;
    }
  }
};

__device__ __forceinline__ float4 ldg4(const float* p) { return __ldg(reinterpret_cast<const float4*>(p)); }
__device__ __forceinline__ float4 ldcs4(const float* p) { return __ldcs(reinterpret_cast<const float4*>(p)); }
// T_{n-1} is read once: keep it out of L1, which holds the gathered T_n rows
__device__ __forceinline__ float4 ld_once4(const float* p) {
  float4 r;
  asm volatile("ld.global.nc.L1::no_allocate.v4.f32 {%0, %1, %2, %3}, [%4];"
               : "=f"(r.x), "=f"(r.y), "=f"(r.z), "=f"(r.w)
               : "l"(p));
  return r;
}


// T_{n+1} (and D T_n) rows are not read again by the launch that writes them:
// their stores keep out of L1, which holds the gathered T_n rows
__device__ __forceinline__ void st_na4(float* p, const float4& v) {
  asm volatile("st.global.L1::no_allocate.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(p), "f"(v.x), "f"(v.y), "f"(v.z),
               "f"(v.w)
               : "memory");
}

// Complex H: the lane's 4 columns are two complex numbers (re, im, re, im); a
// slot's values are a + ib per row (a from the value panel, b from the
// imaginary panel): y += (a + ib)(x_re + i x_im).
struct PanelAccCpx {
  float a[4][4];
  __device__ __forceinline__ void zero() {
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
      for (int c = 0; c < 4; ++c) a[r][c] = 0.f;
  }
  __device__ __forceinline__ void add(const float4& x, const float4& v, const float4& w) {
    const float re[4] = {v.x, v.y, v.z, v.w}, im[4] = {w.x, w.y, w.z, w.w};
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      a[r][0] += re[r] * x.x - im[r] * x.y;
      a[r][1] += re[r] * x.y + im[r] * x.x;
      a[r][2] += re[r] * x.z - im[r] * x.w;
      a[r][3] += re[r] * x.w + im[r] * x.z;
    }
  }
  __device__ __forceinline__ void get(float (&o)[4][4]) const {
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
      for (int c = 0; c < 4; ++c) o[r][c] = a[r][c];
  }
};
