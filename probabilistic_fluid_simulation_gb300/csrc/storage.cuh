// Storage types of planar fields: float (the reference's arithmetic), and the
// 16-bit forms bf16 / fp16 (stored 16-bit, computed in FP32). A lane moves four
// consecutive cells of a row as one vector: 16 bytes for float, 8 for 16-bit.
#pragma once

#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

namespace pfs {

template <typename T>
struct Store;

template <>
struct Store<float> {
    using Vec = float4;  // four cells
    static constexpr int vec_bytes = 16;
    __device__ __forceinline__ static float4 to_f4(const Vec &v) { return v; }
    __device__ __forceinline__ static Vec from_f4(const float4 &f) { return f; }
    __device__ __forceinline__ static float to_f(float x) { return x; }
    __device__ __forceinline__ static float from_f(float x) { return x; }
};

template <>
struct Store<__nv_bfloat16> {
    using Vec = uint2;
    static constexpr int vec_bytes = 8;
    __device__ __forceinline__ static float4 to_f4(const Vec &v)
    {
        const float2 a = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162 *>(&v.x));
        const float2 b = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162 *>(&v.y));
        return make_float4(a.x, a.y, b.x, b.y);
    }
    __device__ __forceinline__ static Vec from_f4(const float4 &f)
    {
        const __nv_bfloat162 a = __float22bfloat162_rn(make_float2(f.x, f.y));
        const __nv_bfloat162 b = __float22bfloat162_rn(make_float2(f.z, f.w));
        Vec v;
        v.x = *reinterpret_cast<const unsigned *>(&a);
        v.y = *reinterpret_cast<const unsigned *>(&b);
        return v;
    }
    __device__ __forceinline__ static float to_f(__nv_bfloat16 x) { return __bfloat162float(x); }
    __device__ __forceinline__ static __nv_bfloat16 from_f(float x) { return __float2bfloat16_rn(x); }
};

template <>
struct Store<__half> {
    using Vec = uint2;
    static constexpr int vec_bytes = 8;
    __device__ __forceinline__ static float4 to_f4(const Vec &v)
    {
        const float2 a = __half22float2(*reinterpret_cast<const __half2 *>(&v.x));
        const float2 b = __half22float2(*reinterpret_cast<const __half2 *>(&v.y));
        return make_float4(a.x, a.y, b.x, b.y);
    }
    __device__ __forceinline__ static Vec from_f4(const float4 &f)
    {
        const __half2 a = __float22half2_rn(make_float2(f.x, f.y));
        const __half2 b = __float22half2_rn(make_float2(f.z, f.w));
        Vec v;
        v.x = *reinterpret_cast<const unsigned *>(&a);
        v.y = *reinterpret_cast<const unsigned *>(&b);
        return v;
    }
    __device__ __forceinline__ static float to_f(__half x) { return __half2float(x); }
    __device__ __forceinline__ static __half from_f(float x) { return __float2half_rn(x); }
};

}  // namespace pfs
