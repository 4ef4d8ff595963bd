// Device-side collision checking for sm_103a: one configuration per thread, grouped into
// segments of W consecutive lanes that stand for one SIMD block of the reference.
//
// The reference checks W configurations at once in SIMD registers (W = 8 with AVX2, 4 with NEON)
// and takes some decisions for the whole block (src/impl/vamp/collision/validity.hh:47-150,
// src/impl/vamp/robots/panda.hh:5630-10259):
//   * a primitive loop stops only when every lane of the block allows it;
//   * a test reports a collision when any lane's test value is negative;
//   * a coarse link sphere that hits in any lane runs the fine tests for every lane.
// Here those block decisions are warp votes restricted to a segment (__ballot_sync plus bit
// tricks), and all control flow is warp-uniform: the four 8-lane segments of a warp run the
// union of their loops, each segment keeping only its own outcomes.  W = 1 gives the reference's
// single-configuration semantics (its validate() broadcasts one configuration to all lanes).
//
// All floating-point operations use explicit round-to-nearest intrinsics so that results are
// bit-identical with the CPU oracle, which performs the same operations in the same order.
#pragma once

#include <cstdint>

namespace vg
{
    constexpr unsigned kFull = 0xffffffffu;

    enum SqrtMode : int
    {
        kSqrtX86 = 0,   // reference built for x86-64: sqrt(v) = v * RSQRTPS(v) (vector/avx.hh:412-415)
        kSqrtExact = 1  // reference built for Arm: correctly rounded sqrt (vector/neon.hh:520-523)
    };

    // ------------------------------------------------------------------ segment-wide votes

    // For each W-lane segment: all bits set if any bit of the segment is set in b.
    template <int W>
    __device__ __forceinline__ unsigned seg_any(unsigned b)
    {
        if constexpr (W == 1)
        {
            return b;
        }
        else if constexpr (W == 32)
        {
            return b ? kFull : 0u;
        }
        else if constexpr (W == 8)
        {
            const unsigned hi = ((b & 0x7f7f7f7fu) + 0x7f7f7f7fu) | b;  // top bit of each byte: byte != 0
            return ((hi & 0x80808080u) >> 7) * 0xffu;
        }
        else if constexpr (W == 4)
        {
            const unsigned hi = ((b & 0x77777777u) + 0x77777777u) | b;  // top bit of each nibble
            return ((hi & 0x88888888u) >> 3) * 0xfu;
        }
        else if constexpr (W == 2)
        {
            const unsigned hi = (b | (b >> 1)) & 0x55555555u;
            return hi * 3u;
        }
        else if constexpr (W == 16)
        {
            return ((b & 0xffffu) ? 0xffffu : 0u) | ((b >> 16) ? 0xffff0000u : 0u);
        }
    }

    template <int W>
    __device__ __forceinline__ unsigned seg_all(unsigned b)
    {
        return ~seg_any<W>(~b);
    }

    // ---------------------------------------------------------------- scalar arithmetic

    __device__ __forceinline__ int signbit_set(float v)
    {
        return __float_as_uint(v) >> 31;
    }

    // max(v, 0) and clamp(v, 0, 1) with the x86 MAXPS/MINPS operand rule (the second operand is
    // returned when the comparison fails), as the reference's vector max/clamp compute them.
    __device__ __forceinline__ float max0(float v)
    {
        return v > 0.0f ? v : 0.0f;
    }

    __device__ __forceinline__ float clamp01(float v)
    {
        const float m = v > 0.0f ? v : 0.0f;
        return m < 1.0f ? m : 1.0f;
    }

    // sin with the Cephes single-precision method (S. L. Moshier, Cephes Math Library sinf.c),
    // which the reference uses (vector/avx.hh:456-544); cos(x) = sin(x + pi/2) with arguments
    // >= pi wrapped by 2 pi (vector/interface.hh:451-458).
    __device__ __forceinline__ float sin_ref(float x)
    {
        unsigned sign = __float_as_uint(x) & 0x80000000u;
        const float ax = fabsf(x);
        int j = __float2int_rn(__fmul_rn(ax, 1.27323954473516f));
        j = (j + 1) & ~1;
        const float yj = __int2float_rn(j);
        sign ^= static_cast<unsigned>(j & 4) << 29;
        float r = __fmaf_rn(yj, -0.78515625f, ax);
        r = __fmaf_rn(yj, -2.4187564849853515625e-4f, r);
        r = __fmaf_rn(yj, -3.77489497744594108e-8f, r);
        const float z = __fmul_rn(r, r);

        float c = __fmaf_rn(2.443315711809948e-5f, z, -1.388731625493765e-3f);
        c = __fmaf_rn(c, z, 4.166664568298827e-2f);
        c = __fmul_rn(c, z);
        c = __fmul_rn(c, z);
        c = __fmaf_rn(-0.5f, z, c);
        c = __fadd_rn(c, 1.0f);

        float s = __fmaf_rn(-1.9515295891e-4f, z, 8.3321608736e-3f);
        s = __fmaf_rn(s, z, -1.6666654611e-1f);
        s = __fmul_rn(s, z);
        s = __fmaf_rn(s, r, r);

        const float y = (j & 2) == 0 ? s : c;
        return __uint_as_float(__float_as_uint(y) ^ sign);
    }

    __device__ __forceinline__ float cos_ref(float x)
    {
        float v = __fadd_rn(x, 1.5707963705062866f);
        if (v >= 3.14159265359f)
        {
            v = __fsub_rn(v, 6.2831854820251465f);
        }
        return sin_ref(v);
    }

    __device__ __forceinline__ void vg_sincos_ref(float x, float *s, float *c)
    {
        *s = sin_ref(x);
        *c = cos_ref(x);
    }

    // x86 RSQRTPS, from the 2048-entry table of its results on [1, 4): the result depends only on
    // the exponent parity and the top 10 mantissa bits and scales by powers of four.
    // Valid for normal positive inputs.
    __device__ __forceinline__ float rsqrt_x86(const uint32_t *tab, float v)
    {
        const unsigned u = __float_as_uint(v);
        const int E = static_cast<int>(u >> 23) - 127;
        const int odd = E & 1;
        const int k = (E - odd) >> 1;
        const unsigned tb = __ldg(tab + ((static_cast<unsigned>(odd) << 10) | ((u >> 13) & 1023u)));
        return __uint_as_float((static_cast<unsigned>(static_cast<int>(tb >> 23) - k) << 23) | (tb & 0x7fffffu));
    }

    // ------------------------------------------------------------------ environment view

    // Record layouts in shared memory (float4 aligned); min_distance is where the primitive loop
    // reads it first.
    //   sphere   (2 x float4): x y z r | min_d . . .
    //   capsule  (3 x float4): x1 y1 z1 xv | yv zv r rdv | min_d . . .
    //   cuboid   (4 x float4): x y z r1 | a1x a1y a1z r2 | a2x a2y a2z r3 | a3x a3y a3z min_d
    __host__ __device__ constexpr int rec_f4(int kind)
    {
        return kind == 0 ? 2 : (kind <= 2 ? 3 : 4);
    }

    __host__ __device__ constexpr int min_d_offset(int kind)
    {
        return kind == 0 ? 4 : (kind <= 2 ? 8 : 15);
    }

    // One pointcloud's CAPT on the device: the query tables built from the reference layout
    // (collision/capt.hh:584-617) by vg_capt_ring.cu.  Split values three tree levels per node
    // (2 float4: the subtree's 7 values in heap order, then a pad) in groups of 2^rem * 8^g
    // nodes; per leaf its box and first block (2 float4); per leaf and ring the end of the
    // blocks up to that ring; the 8-point blocks (x[8] y[8] z[8] = 6 float4), each leaf's
    // nearest ring first.
    constexpr int kCaptRings = 32;
    struct CaptView
    {
        const float4 *nodes;
        const float4 *leaves;
        const uint32_t *ends;
        const float4 *aff;
        float top[6];
        float r_point;
        int nlog2;
        float top_tests[3];  // the rem = nlog2 mod 3 levels above the first group, heap order
        int rem;
        int groups;          // nlog2 / 3
        int pad[3];
        float ring_edge[kCaptRings];  // lower edge of each distance ring, rounded down
    };
    constexpr int kMaxClouds = 4;

    // One heightfield (collision/shapes.hh:250-311) on the device: offsets, inverted scales
    // (collision/factory.hh:376-385), grid size, samples [xd * yd] in global memory, and its
    // insertion id (debug reports).
    struct HeightView
    {
        float x, y, z, xs, ys, zs;
        int xd, yd;
        const float *data;
        int id;
        int pad;
    };
    constexpr int kMaxHeightfields = 8;

    struct EnvView
    {
        const float4 *rec[5];
        int n[5];
        const uint32_t *rsqrt_tab;
        int sqrt_mode;
        const CaptView *clouds;
        int n_clouds;
        const float4 *att;  // attachment: 3 transform rows {R[r][0..2], t[r]}, then spheres
        int n_att;          // -1: none
        const HeightView *hf;
        int n_hf;
    };

    // sphere_heightfield (collision/sphere_heightfield.hh:9-30), sign bit set iff the sphere is
    // below the surface: the cell floor(clamp(xs * (x0 - x) + xd / 2, 0, xd)) (one fused
    // multiply-add) and the same in y, index y * xd + x, and the value z - r - (zs * h + z0) as
    // the reference's x86-64 build reassociates it, fma(-zs, h, (z - r) - z0).  Centres beyond
    // the far edges (where the reference reads past its samples) use the last cell.
    __device__ __forceinline__ float t_heightfield(const HeightView &h, float x, float y, float z, float r)
    {
        const float fx = __fmaf_rn(h.xs, __fsub_rn(h.x, x), static_cast<float>(h.xd / 2));
        const float fy = __fmaf_rn(h.ys, __fsub_rn(h.y, y), static_cast<float>(h.yd / 2));
        const float mx = fx > 0.0f ? fx : 0.0f, my = fy > 0.0f ? fy : 0.0f;  // max(v, 0), NaN to 0
        const float cx = floorf(mx < static_cast<float>(h.xd) ? mx : static_cast<float>(h.xd));
        const float cy = floorf(my < static_cast<float>(h.yd) ? my : static_cast<float>(h.yd));
        long long idx = static_cast<long long>(__fmaf_rn(cy, static_cast<float>(h.xd), cx));
        const long long last = static_cast<long long>(h.xd) * h.yd - 1;
        idx = idx < 0 ? 0 : (idx > last ? last : idx);
        return __fmaf_rn(-h.zs, __ldg(h.data + idx), __fsub_rn(__fsub_rn(z, r), h.z));
    }

    __device__ __forceinline__ float sql2(float ax, float ay, float az, float bx, float by, float bz)
    {
        const float dx = __fsub_rn(ax, bx), dy = __fsub_rn(ay, by), dz = __fsub_rn(az, bz);
        return __fmaf_rn(dz, dz, __fmaf_rn(dy, dy, __fmul_rn(dx, dx)));
    }

    // Primitive tests: sign bit set iff the sphere collides (collision/sphere_*.hh).
    __device__ __forceinline__ float t_sphere(const float4 *o, float x, float y, float z, float r)
    {
        const float4 a = o[0];
        const float rs = __fadd_rn(a.w, r);
        return __fmaf_rn(-rs, rs, sql2(a.x, a.y, a.z, x, y, z));
    }

    __device__ __forceinline__ float t_capsule(const float4 *o, float x, float y, float z, float r)
    {
        const float4 a = o[0], b = o[1];  // x1 y1 z1 xv | yv zv r rdv
        const float dot = __fmaf_rn(__fsub_rn(z, a.z), b.y, __fmaf_rn(__fsub_rn(y, a.y), b.x, __fmul_rn(__fsub_rn(x, a.x), a.w)));
        const float t = clamp01(__fmul_rn(dot, b.w));
        const float px = __fmaf_rn(a.w, t, a.x), py = __fmaf_rn(b.x, t, a.y), pz = __fmaf_rn(b.y, t, a.z);
        const float rs = __fadd_rn(r, b.z);
        return __fmaf_rn(-rs, rs, sql2(x, y, z, px, py, pz));
    }

    __device__ __forceinline__ float t_zcapsule(const float4 *o, float x, float y, float z, float r)
    {
        const float4 a = o[0], b = o[1];
        const float t = clamp01(__fmul_rn(__fmul_rn(__fsub_rn(z, a.z), b.y), b.w));
        const float pz = __fmaf_rn(b.y, t, a.z);
        const float rs = __fadd_rn(r, b.z);
        return __fmaf_rn(-rs, rs, sql2(x, y, z, a.x, a.y, pz));
    }

    __device__ __forceinline__ float t_cuboid(const float4 *o, float x, float y, float z, float rsq)
    {
        const float4 a = o[0], b = o[1], c = o[2], d = o[3];
        // a: x y z r1 | b: a1x a1y a1z r2 | c: a2x a2y a2z r3 | d: a3x a3y a3z min_d
        const float xs = __fsub_rn(x, a.x), ys = __fsub_rn(y, a.y), zs = __fsub_rn(z, a.z);
        const float a1 = max0(__fsub_rn(fabsf(__fmaf_rn(b.z, zs, __fmaf_rn(b.y, ys, __fmul_rn(b.x, xs)))), a.w));
        const float a2 = max0(__fsub_rn(fabsf(__fmaf_rn(c.z, zs, __fmaf_rn(c.y, ys, __fmul_rn(c.x, xs)))), b.w));
        const float a3 = max0(__fsub_rn(fabsf(__fmaf_rn(d.z, zs, __fmaf_rn(d.y, ys, __fmul_rn(d.x, xs)))), c.w));
        return __fsub_rn(__fmaf_rn(a3, a3, __fmaf_rn(a2, a2, __fmul_rn(a1, a1))), rsq);
    }

    __device__ __forceinline__ float t_zcuboid(const float4 *o, float x, float y, float z, float rsq)
    {
        const float4 a = o[0], b = o[1], c = o[2];
        const float xs = __fsub_rn(x, a.x), ys = __fsub_rn(y, a.y), zs = __fsub_rn(z, a.z);
        const float a1 = max0(__fsub_rn(fabsf(__fmaf_rn(b.y, ys, __fmul_rn(b.x, xs))), a.w));
        const float a2 = max0(__fsub_rn(fabsf(__fmaf_rn(c.y, ys, __fmul_rn(c.x, xs))), b.w));
        const float a3 = max0(__fsub_rn(fabsf(zs), c.w));
        return __fsub_rn(__fmaf_rn(a3, a3, __fmaf_rn(a2, a2, __fmul_rn(a1, a1))), rsq);
    }

    // The early-exit bound max_extent = |c| + r of one lane (validity.hh:56): +inf when the
    // lane can never allow a stop (|c|^2 zero or subnormal under the x86 rule).
    __device__ __forceinline__ float max_extent(const EnvView &e, float v, float r)
    {
        if (e.sqrt_mode == kSqrtX86)
        {
            return v >= 1.17549435e-38f ? __fmaf_rn(v, rsqrt_x86(e.rsqrt_tab, v), r) : __int_as_float(0x7f800000);
        }
        return __fadd_rn(__fsqrt_rn(v), r);
    }

    // max over the W lanes of a segment (segments are aligned groups of W lanes)
    template <int W>
    __device__ __forceinline__ float seg_max(float v)
    {
#pragma unroll
        for (int o = 1; o < W; o <<= 1)
        {
            v = fmaxf(v, __shfl_xor_sync(kFull, v, o));
        }
        return v;
    }

    __device__ __forceinline__ float warp_max(float v)
    {
#pragma unroll
        for (int o = 1; o < 32; o <<= 1)
        {
            v = fmaxf(v, __shfl_xor_sync(kFull, v, o));
        }
        return v;
    }

    template <int KIND>
    __device__ __forceinline__ float prim_test(const float4 *o, float x, float y, float z, float r, float rsq)
    {
        if constexpr (KIND == 0)
            return t_sphere(o, x, y, z, r);
        else if constexpr (KIND == 1)
            return t_capsule(o, x, y, z, r);
        else if constexpr (KIND == 2)
            return t_zcapsule(o, x, y, z, r);
        else if constexpr (KIND == 3)
            return t_cuboid(o, x, y, z, rsq);
        else
            return t_zcuboid(o, x, y, z, rsq);
    }

    // One kind's sorted primitive list against NS query spheres.
    //
    // The reference walks the list per sphere and stops at the first object whose min_distance
    // minus max_extent has a clear sign bit in every lane of the block.  Since min_distance is
    // sorted and rounding is monotone, that stop is the first object with min_distance >= M, M
    // being the largest max_extent over the block's lanes; the objects before it are tested and a
    // collision is any lane's test with its sign bit set.  Here each object record is read once
    // for the NS spheres; sphere s tests it while min_distance < Mw[s] (the warp's largest M for
    // that sphere, a uniform branch) and counts the result only while min_distance < M[s] (its
    // own segment's bound).  Sign bits are OR-ed into bits[]; the segment vote happens once.
    template <int KIND, int NS>
    __device__ __forceinline__ void kind_pass(
        const EnvView &e, float Mall, const float *Mw, const float *M, const float *x, const float *y,
        const float *z, const float *r, const float *rsq, unsigned *bits)
    {
        const float4 *rec = e.rec[KIND];
        const int n = e.n[KIND];
#pragma unroll 1
        for (int i = 0; i < n; ++i)
        {
            const float4 *o = rec + i * rec_f4(KIND);
            const float md = reinterpret_cast<const float *>(o)[min_d_offset(KIND)];
            if (!(md < Mall))
            {
                break;
            }
#pragma unroll
            for (int s = 0; s < NS; ++s)
            {
                if (md < Mw[s])
                {
                    const float t = prim_test<KIND>(o, x[s], y[s], z[s], r[s], rsq[s]);
                    bits[s] |= md < M[s] ? __float_as_uint(t) : 0u;
                }
            }
        }
    }

#ifndef VG_CAPT_SHARED_WEIGHT
#define VG_CAPT_SHARED_WEIGHT 4
#endif

    // CAPT::collides_simd (collision/capt.hh:425-506), per lane.  The reference's block result
    // is the OR over its lanes; its early exits (no lane in the top box, no lane in its leaf box)
    // return false for exactly the lanes that would not hit, so the per-lane form is the same
    // test.  capt_locate does the box tests and the descent: the lane's sphere must be compared
    // with the points of affordance blocks [b0, b1) (empty: it cannot hit), radius^2 rc.
    __device__ __forceinline__ void capt_locate(const CaptView &c, float x, float y, float z, float r, uint32_t &b0,
                                                uint32_t &b1, float &rc)
    {
        b0 = b1 = 0;
        const float rad = __fadd_rn(r, c.r_point);
        rc = __fmul_rn(rad, rad);
        const float p[3] = {x, y, z};
        bool in = true;
#pragma unroll
        for (int k = 0; k < 3; ++k)
        {
            in &= (__fadd_rn(p[k], rad) >= c.top[k]) & (__fsub_rn(p[k], rad) <= c.top[3 + k]);
        }
        if (!in)
        {
            return;
        }
        // the last ring whose lower edge is within the sphere's reach (the margin dwarfs the FP32
        // error of the point test); independent of the descent
        const float reach = fabsf(rad);
        const float lim = __fmaf_rn(reach, 1e-5f, reach);
        int ring = 0;
#pragma unroll
        for (int s = kCaptRings / 2; s > 0; s >>= 1)
        {
            ring += c.ring_edge[ring + s] <= lim ? s : 0;
        }
        // descent (right child: coordinate >= split value; level i splits axis i mod 3): the
        // levels above the first group one at a time, then three levels per node
        uint32_t node = 0;
        if (c.rem > 0)
        {
            const int r0 = x >= c.top_tests[0] ? 1 : 0;
            node = r0;
            if (c.rem > 1)
            {
                node = 2 * node + (y >= c.top_tests[1 + r0] ? 1 : 0);
            }
        }
        const float q0 = c.rem == 0 ? x : (c.rem == 1 ? y : z);
        const float q1 = c.rem == 0 ? y : (c.rem == 1 ? z : x);
        const float q2 = c.rem == 0 ? z : (c.rem == 1 ? x : y);
        const float4 *group = c.nodes;
        uint32_t size = 1u << c.rem;
#pragma unroll 1
        for (int g = 0; g < c.groups; ++g)
        {
            const float4 t0 = __ldg(group + 2 * node), t1 = __ldg(group + 2 * node + 1);
            const uint32_t c0 = q0 >= t0.x ? 1u : 0u;
            const uint32_t c1 = q1 >= (c0 ? t0.z : t0.y) ? 1u : 0u;
            const float t2 = c0 ? (c1 ? t1.z : t1.y) : (c1 ? t1.x : t0.w);
            const uint32_t c2 = q2 >= t2 ? 1u : 0u;
            node = 8u * node + 4u * c0 + 2u * c1 + c2;
            group += 2 * static_cast<size_t>(size);
            size *= 8u;
        }
        const float4 l0 = __ldg(c.leaves + 2 * static_cast<size_t>(node)), l1 = __ldg(c.leaves + 2 * static_cast<size_t>(node) + 1);
        const uint32_t end = __ldg(c.ends + static_cast<size_t>(node) * kCaptRings + ring);
        const float lo[3] = {l0.x, l0.y, l0.z}, hi[3] = {l0.w, l1.x, l1.y};
        float d[3];
#pragma unroll
        for (int j = 0; j < 3; ++j)
        {
            const float m = p[j] > lo[j] ? p[j] : lo[j];
            const float cl = m < hi[j] ? m : hi[j];
            d[j] = __fsub_rn(p[j], cl);
        }
        if (!(__fmaf_rn(d[2], d[2], __fmaf_rn(d[1], d[1], __fmul_rn(d[0], d[0]))) <= rc))
        {
            return;
        }
        b0 = __float_as_uint(l1.z);
        b1 = end;
    }

    // Whether any of the 8 points of affordance block b lies within sqrt(rc) of (x, y, z).
    __device__ __forceinline__ bool capt_block(const CaptView &c, uint32_t b, float x, float y, float z, float rc)
    {
        const float4 *blk = c.aff + 6 * static_cast<size_t>(b);
        const float4 xs0 = __ldg(blk + 0), xs1 = __ldg(blk + 1), ys0 = __ldg(blk + 2), ys1 = __ldg(blk + 3);
        const float4 zs0 = __ldg(blk + 4), zs1 = __ldg(blk + 5);
        const float ax[8] = {xs0.x, xs0.y, xs0.z, xs0.w, xs1.x, xs1.y, xs1.z, xs1.w};
        const float ay[8] = {ys0.x, ys0.y, ys0.z, ys0.w, ys1.x, ys1.y, ys1.z, ys1.w};
        const float az[8] = {zs0.x, zs0.y, zs0.z, zs0.w, zs1.x, zs1.y, zs1.z, zs1.w};
        bool hit = false;
#pragma unroll
        for (int j = 0; j < 8; ++j)
        {
            const float dx = __fsub_rn(ax[j], x), dy = __fsub_rn(ay[j], y), dz = __fsub_rn(az[j], z);
            hit |= __fmaf_rn(dz, dz, __fmaf_rn(dy, dy, __fmul_rn(dx, dx))) <= rc;
        }
        return hit;
    }

    // The CAPT query of every lane with `ask`, as a ballot of the lanes that hit.  Each lane's
    // answer is the OR over the points of its affordance blocks, whoever scans them: when one
    // lane's list is long compared with the warp's total (a tree built for large spheres affords
    // thousands of points per leaf), the whole warp scans each lane's list in turn, 32 blocks at a
    // time, instead of every lane walking its own.  Warp-uniform; all 32 lanes must call.
    static __device__ __noinline__ unsigned capt_warp(const CaptView &c, float x, float y, float z, float r, bool ask)
    {
        const int lane = threadIdx.x & 31;
        uint32_t b0 = 0, b1 = 0;
        float rc = 0.0f;
        if (ask)
        {
            capt_locate(c, x, y, z, r, b0, b1, rc);
        }
        const uint32_t len = b1 - b0;
        const uint32_t longest = __reduce_max_sync(kFull, len);
        if (longest == 0)
        {
            return 0u;
        }
        // warp iterations: each lane its own list (longest), or the lists one after another, 32
        // blocks per step (a shared step also pays broadcasts and a vote: weighted by
        // VG_CAPT_SHARED_WEIGHT / 4)
        const uint32_t shared_steps = __reduce_add_sync(kFull, (len + 31u) >> 5);
        bool hit = false;
        if (4u * longest <= VG_CAPT_SHARED_WEIGHT * shared_steps)
        {
            // two blocks per step: their loads overlap
#pragma unroll 1
            for (uint32_t b = b0; b < b1 && !hit; b += 2)
            {
                hit = capt_block(c, b, x, y, z, rc) | (b + 1 < b1 && capt_block(c, b + 1, x, y, z, rc));
            }
        }
        else
        {
            unsigned pending = __ballot_sync(kFull, len > 0);
#pragma unroll 1
            while (pending)
            {
                const int L = __ffs(pending) - 1;
                pending &= pending - 1u;
                const float qx = __shfl_sync(kFull, x, L), qy = __shfl_sync(kFull, y, L), qz = __shfl_sync(kFull, z, L);
                const float qrc = __shfl_sync(kFull, rc, L);
                const uint32_t s0 = __shfl_sync(kFull, b0, L), s1 = __shfl_sync(kFull, b1, L);
                bool found = false;
#pragma unroll 1
                for (uint32_t base = s0; base < s1; base += 32u)
                {
                    const uint32_t b = base + static_cast<uint32_t>(lane);
                    const bool h = b < s1 && capt_block(c, b, qx, qy, qz, qrc);
                    if (__any_sync(kFull, h))
                    {
                        found = true;
                        break;
                    }
                }
                if (lane == L)
                {
                    hit = found;
                }
            }
        }
        return __ballot_sync(kFull, hit);
    }

    // sphere_environment_in_collision (validity.hh:47-150) for NS spheres at once, each over the
    // segments in `mask`.  hit[s] receives the lanes of the segments whose block collides for
    // sphere s.  Warp-uniform; all 32 lanes must call.
    // kExt: also the heightfields (kernels built for environments with heightfields or an
    // attachment; the default kernels leave them out)
    template <int W, int NS, bool kExt = false>
    __device__ __forceinline__ void env_multi(const EnvView &e, const float4 *sph, unsigned mask, unsigned *hit)
    {
        const int lane = threadIdx.x & 31;
        const bool on = (mask >> lane) & 1u;
        float x[NS], y[NS], z[NS], r[NS], rsq[NS], M[NS], Mw[NS];
        unsigned bits[NS];
        float Mall = -__int_as_float(0x7f800000);
#pragma unroll
        for (int s = 0; s < NS; ++s)
        {
            const float4 c = sph[s];
            x[s] = c.x;
            y[s] = c.y;
            z[s] = c.z;
            r[s] = c.w;
            rsq[s] = __fmul_rn(c.w, c.w);
            const float v = __fmaf_rn(c.x, c.x, __fmaf_rn(c.z, c.z, __fmul_rn(c.y, c.y)));
            const float m = seg_max<W>(max_extent(e, v, c.w));
            M[s] = on ? m : -__int_as_float(0x7f800000);
            // max_extent is >= 0 (or +inf): as unsigned integers its bit patterns order like the
            // floats, so one warp reduction gives the warp-wide bound (inactive lanes count as 0)
            Mw[s] = __uint_as_float(__reduce_max_sync(kFull, on ? __float_as_uint(m) : 0u));
            Mall = fmaxf(Mall, Mw[s]);
            bits[s] = 0u;
        }
        kind_pass<0, NS>(e, Mall, Mw, M, x, y, z, r, rsq, bits);
        kind_pass<1, NS>(e, Mall, Mw, M, x, y, z, r, rsq, bits);
        kind_pass<2, NS>(e, Mall, Mw, M, x, y, z, r, rsq, bits);
        kind_pass<3, NS>(e, Mall, Mw, M, x, y, z, r, rsq, bits);
        kind_pass<4, NS>(e, Mall, Mw, M, x, y, z, r, rsq, bits);
        if constexpr (kExt)
        {
#pragma unroll 1
            for (int h = 0; h < e.n_hf; ++h)
            {
#pragma unroll
                for (int s = 0; s < NS; ++s)
                {
                    bits[s] |= __float_as_uint(t_heightfield(e.hf[h], x[s], y[s], z[s], r[s]));
                }
            }
        }
#pragma unroll
        for (int s = 0; s < NS; ++s)
        {
            hit[s] = seg_any<W>(__ballot_sync(kFull, bits[s] >> 31)) & mask;
        }
        // pointclouds, for the blocks the primitives did not already put in collision
#pragma unroll 1
        for (int c = 0; c < e.n_clouds; ++c)
        {
#pragma unroll
            for (int s = 0; s < NS; ++s)
            {
                const bool ask = on && !((hit[s] >> lane) & 1u);
                if (__any_sync(kFull, ask))
                {
                    hit[s] |= seg_any<W>(capt_warp(e.clouds[c], x[s], y[s], z[s], r[s], ask)) & mask;
                }
            }
        }
    }

    // A frame as 12 floats: R row-major, then t.
    struct Frame
    {
        float m[12];
    };

    // t + R o for a point offset o (o.w, the radius, is passed through): t, then one fused
    // multiply-add per column of R, for every coordinate (the generated kinematics' order).
    __device__ __forceinline__ float4 frame_point(const Frame &f, const float4 o)
    {
        float c[3];
#pragma unroll
        for (int r = 0; r < 3; ++r)
        {
            float acc = f.m[9 + r];
            acc = __fmaf_rn(f.m[3 * r + 0], o.x, acc);
            acc = __fmaf_rn(f.m[3 * r + 1], o.y, acc);
            acc = __fmaf_rn(f.m[3 * r + 2], o.z, acc);
            c[r] = acc;
        }
        return make_float4(c[0], c[1], c[2], o.w);
    }

    // Single-sphere query, inlined into the caller.
    template <int W, bool kExt = false>
    __device__ __forceinline__ unsigned env_query_inline(const EnvView &e, float x, float y, float z, float r, unsigned mask)
    {
        const float4 s = make_float4(x, y, z, r);
        unsigned hit;
        env_multi<W, 1, kExt>(e, &s, mask, &hit);
        return hit;
    }

    // Single-sphere form.
    template <int W, bool kExt = false>
    __device__ __noinline__ unsigned env_query(const EnvView &e, float x, float y, float z, float r, unsigned mask)
    {
        const float4 s = make_float4(x, y, z, r);
        unsigned hit;
        env_multi<W, 1, kExt>(e, &s, mask, &hit);
        return hit;
    }

    // Fine tests of one link's NS spheres (one function per distinct NS): the segments in `mask`
    // whose block collides for any of the spheres.
    template <int W, int NS, bool kExt = false>
    __device__ __noinline__ unsigned env_any(const EnvView &e, const float4 *sph, unsigned mask)
    {
        unsigned hit[NS];
        env_multi<W, NS, kExt>(e, sph, mask, hit);
        unsigned any = 0;
#pragma unroll
        for (int s = 0; s < NS; ++s)
        {
            any |= hit[s];
        }
        return any;
    }

    // sphere_sphere_self_collision (validity.hh:23-44) for the segments in `mask`.
    template <int W>
    __device__ __forceinline__ unsigned self_query(
        float ax, float ay, float az, float ar, float bx, float by, float bz, float br, unsigned mask)
    {
        const float rs = __fadd_rn(ar, br);
        const float t = __fmaf_rn(-rs, rs, sql2(ax, ay, az, bx, by, bz));
        return seg_any<W>(__ballot_sync(kFull, signbit_set(t))) & mask;
    }

    // Sign bit of one fine self-collision test, for OR-accumulation; rs is the pair's radius sum.
    __device__ __forceinline__ unsigned self_bits(float ax, float ay, float az, float bx, float by, float bz, float rs)
    {
        return __float_as_uint(__fmaf_rn(-rs, rs, sql2(ax, ay, az, bx, by, bz)));
    }

    // Threads per block of every checking kernel, and the stride of the per-thread columns of
    // the robots' shared-memory stage.
    constexpr int kStageStride = 128;
    // words of per-warp shared scratch available to a generated fkcc (environment checks per robot)
    constexpr int kWarpScratch = 64;

    // The context a generated Robot::fkcc body runs against.  kExt: the environment queries also
    // test heightfields.  kOrdered: the warp's segments are consecutive blocks of one edge in the
    // reference's order (the same-edge schedule), so only the first colliding segment decides the
    // edge's verdict and block count.
    template <int W, bool kExtended = false, bool kOrdered = false>
    struct CheckCtx
    {
        static constexpr int kW = W;
        static constexpr bool kExt = kExtended;
        const EnvView &env;
        unsigned alive;
        // every active lane's configuration lies inside the joint limits widened by the culling
        // slack: fine self pairs proven unable to collide there may be skipped
        bool in_limits = false;
        // this thread's column of the robot's shared-memory stage: element i at stage[i * kStageStride]
        float *stage = nullptr;
        // this warp's scratch (kWarpScratch words) for warp-uniform values such as per-link hit masks
        unsigned *wsc = nullptr;

        // inlined at each call site: the table-driven robot forms call it from two places (coarse
        // and fine spheres), and an out-of-line query costs them more than the second copy
        __device__ __forceinline__ unsigned env_hit(float x, float y, float z, float r, unsigned mask)
        {
            return env_query_inline<W, kExt>(env, x, y, z, r, mask);
        }

        template <int NS>
        __device__ __forceinline__ void env_many(const float4 *s, unsigned mask, unsigned *hit)
        {
            env_multi<W, NS, kExt>(env, s, mask, hit);
        }

        template <int NS>
        __device__ __forceinline__ unsigned env_any_hit(const float4 *s, unsigned mask)
        {
            return env_any<W, NS, kExt>(env, s, mask);
        }

        __device__ __forceinline__ unsigned self_hit(
            float ax, float ay, float az, float ar, float bx, float by, float bz, float br, unsigned mask)
        {
            return self_query<W>(ax, ay, az, ar, bx, by, bz, br, mask);
        }

        // Removes the colliding segments `hit` from alive and returns what is left.  kOrdered:
        // the segments after the first colliding one go too, since no result of theirs can
        // change the verdict or the block count (the first colliding block stays the first).
        __device__ __forceinline__ unsigned kill(unsigned hit)
        {
            if constexpr (kOrdered)
            {
                alive &= hit ? (1u << (__ffs(hit) - 1)) - 1u : kFull;
            }
            else
            {
                alive &= ~hit;
            }
            return alive;
        }

        // the segments in `mask` for which any OR-accumulated sign bit is set
        __device__ __forceinline__ unsigned vote(unsigned bits, unsigned mask)
        {
            return seg_any<W>(__ballot_sync(kFull, bits >> 31)) & mask;
        }
    };

    // Fine environment tests of one link's spheres, in order, for the segments in `need`.
    // Clears colliding segments from ctx.alive; returns true once none is left.
    template <int N, typename Ctx>
    __device__ __forceinline__ bool env_fine(Ctx &ctx, const float4 *s, unsigned need)
    {
#pragma unroll 1
        for (int k = 0; k < N; ++k)
        {
            const float4 c = s[k];
            const unsigned hit = ctx.env_hit(c.x, c.y, c.z, c.w, need);
            if (hit)
            {
                need &= ~hit;
                if (!ctx.kill(hit))
                {
                    return true;
                }
                need &= ctx.alive;
                if (!need)
                {
                    return false;
                }
            }
        }
        return false;
    }

    // Fine self-collision tests of one link pair: every sphere of link A against every sphere
    // of link B (the reference's generated pair list is this cross product), for the segments
    // in `need`.  Clears colliding segments from ctx.alive; returns true once none is left.
    template <int NA, int NB, typename Ctx>
    __device__ __forceinline__ bool self_cross(Ctx &ctx, const float4 *sa, const float4 *sb, unsigned need)
    {
#pragma unroll 1
        for (int i = 0; i < NA; ++i)
        {
            const float4 a = sa[i];
#pragma unroll 1
            for (int j = 0; j < NB; ++j)
            {
                const float4 b = sb[j];
                const unsigned hit = ctx.self_hit(a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w, need);
                if (hit)
                {
                    need &= ~hit;
                    if (!ctx.kill(hit))
                    {
                        return true;
                    }
                    need &= ctx.alive;
                    if (!need)
                    {
                        return false;
                    }
                }
            }
        }
        return false;
    }
}  // namespace vg
