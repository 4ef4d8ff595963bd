// Clearance field of an environment's primitives: a grid over their bounding box (widened by
// 10 cm) whose cells hold a lower bound of the distance from any point of the cell to the
// nearest primitive, as each primitive's collision test measures it:
//   sphere       |x - c| - R
//   capsule      distance to the segment - R (the test's clamped projection is some point of
//                the segment, so its distance is at least this)
//   cuboid       |(max(|a_k . (x - c)| - r_k, 0))_k|, the quantity the test compares with the
//                query radius; L-Lipschitz with L the largest singular value of the axis
//                matrix, bounded above by Gershgorin on A^T A
// Each cell stores min over primitives of (D(centre) - L * h), h the half-diagonal of the cell
// widened by 1e-4 m, rounded down.  A sphere of radius r whose centre lies in a cell with a
// bound above r + 1e-4 m cannot make any primitive test negative (the FP32 error of the tests is
// below 1e-6 m), so the queries skip the primitives for it (vg_check.cuh, field_far).
#include "../../include/vamp_gb300.h"
#include "vg_internal.h"

#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

namespace vg
{
    namespace
    {
        struct FieldPrim
        {
            int kind;     // 0 sphere, 1 capsule, 3 cuboid
            float f[15];  // sphere: c, R; capsule: p1, v, R; cuboid: c, a1, a2, a3, r1..r3
            float lip;    // Lipschitz constant of D
        };

        struct FieldGeom
        {
            double lo[3];
            double cell;
            int dim[3];
        };

        __device__ double prim_distance(const FieldPrim &p, double x, double y, double z)
        {
            const float *f = p.f;
            if (p.kind == 0)
            {
                const double dx = x - f[0], dy = y - f[1], dz = z - f[2];
                return sqrt(dx * dx + dy * dy + dz * dz) - f[3];
            }
            if (p.kind == 1)
            {
                const double vv = static_cast<double>(f[3]) * f[3] + static_cast<double>(f[4]) * f[4] +
                                  static_cast<double>(f[5]) * f[5];
                const double wx = x - f[0], wy = y - f[1], wz = z - f[2];
                double t = vv > 0.0 ? (wx * f[3] + wy * f[4] + wz * f[5]) / vv : 0.0;
                t = t < 0.0 ? 0.0 : (t > 1.0 ? 1.0 : t);
                const double dx = wx - t * f[3], dy = wy - t * f[4], dz = wz - t * f[5];
                return sqrt(dx * dx + dy * dy + dz * dz) - f[6];
            }
            const double wx = x - f[0], wy = y - f[1], wz = z - f[2];
            double s = 0.0;
            for (int k = 0; k < 3; ++k)
            {
                const float *a = f + 3 + 3 * k;
                double d = fabs(wx * a[0] + wy * a[1] + wz * a[2]) - f[12 + k];
                d = d > 0.0 ? d : 0.0;
                s += d * d;
            }
            return sqrt(s);
        }

        __global__ void field_kernel(const FieldPrim *prims, int n, FieldGeom g, float *out)
        {
            const long long cells = static_cast<long long>(g.dim[0]) * g.dim[1] * g.dim[2];
            const long long idx = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
            if (idx >= cells)
                return;
            const long long i = idx % g.dim[0], j = (idx / g.dim[0]) % g.dim[1], k = idx / (static_cast<long long>(g.dim[0]) * g.dim[1]);
            const double x = g.lo[0] + (i + 0.5) * g.cell, y = g.lo[1] + (j + 0.5) * g.cell, z = g.lo[2] + (k + 0.5) * g.cell;
            const double h = sqrt(3.0) * (0.5 * g.cell + 1e-4);
            double lb = 1e30;
            for (int p = 0; p < n; ++p)
            {
                const double d = prim_distance(prims[p], x, y, z) - prims[p].lip * h;
                lb = d < lb ? d : lb;
            }
            out[idx] = __double2float_rd(lb);
        }

        // Gershgorin bound of the largest singular value of the 3x3 matrix with rows a0, a1, a2
        double axis_lipschitz(const double a[3][3])
        {
            double m = 0.0;
            for (int r = 0; r < 3; ++r)
            {
                double row = 0.0;
                for (int c = 0; c < 3; ++c)
                {
                    double g = 0.0;  // (A^T A)[r][c]
                    for (int k = 0; k < 3; ++k)
                        g += a[k][r] * a[k][c];
                    row += std::fabs(g);
                }
                m = std::max(m, row);
            }
            return std::sqrt(m) * (1.0 + 1e-6) + 1e-9;
        }
    }  // namespace

    void EnvField::release()
    {
        if (data)
            cudaFree(data);
        data = nullptr;
    }

    int build_field(const vg_env *e, EnvField &out)
    {
        out.release();
        std::vector<FieldPrim> prims;
        double lo[3] = {1e30, 1e30, 1e30}, hi[3] = {-1e30, -1e30, -1e30};
        auto grow = [&](double c, double ext, int k) {
            lo[k] = std::min(lo[k], c - ext);
            hi[k] = std::max(hi[k], c + ext);
        };
        for (int kind = 0; kind < 5; ++kind)
        {
            const int w = (kind == 0 ? 4 : (kind <= 2 ? 8 : 15)) + 1;
            const std::vector<float> &obj = e->obj[kind];
            for (size_t i = 0; i + w <= obj.size(); i += w)
            {
                const float *f = &obj[i];
                FieldPrim p{};
                p.lip = 1.0f;
                if (kind == 0)
                {
                    p.kind = 0;
                    std::copy(f, f + 4, p.f);
                    for (int k = 0; k < 3; ++k)
                        grow(f[k], f[3], k);
                }
                else if (kind <= 2)
                {
                    // capsule fields x1 y1 z1 xv yv zv r rdv (a z-aligned one has xv = yv = 0)
                    p.kind = 1;
                    std::copy(f, f + 7, p.f);
                    for (int k = 0; k < 3; ++k)
                    {
                        const double a = f[k], b = static_cast<double>(f[k]) + f[3 + k];
                        grow(0.5 * (a + b), 0.5 * std::fabs(b - a) + f[6], k);
                    }
                }
                else
                {
                    // cuboid fields: centre, axis_1, axis_2, axis_3, half extents; the z-aligned
                    // test uses the xy parts of axes 1 and 2 and z itself as axis 3
                    p.kind = 3;
                    std::copy(f, f + 15, p.f);
                    if (kind == 4)
                    {
                        p.f[5] = 0.0f;
                        p.f[8] = 0.0f;
                        p.f[9] = 0.0f;
                        p.f[10] = 0.0f;
                        p.f[11] = 1.0f;
                    }
                    double a[3][3];
                    for (int k = 0; k < 3; ++k)
                        for (int c = 0; c < 3; ++c)
                            a[k][c] = p.f[3 + 3 * k + c];
                    p.lip = static_cast<float>(axis_lipschitz(a) * (1.0 + 1e-6));
                    for (int c = 0; c < 3; ++c)
                    {
                        double ext = 0.0;
                        for (int k = 0; k < 3; ++k)
                            ext += std::fabs(a[k][c]) * p.f[12 + k];
                        grow(p.f[c], ext, c);
                    }
                }
                prims.push_back(p);
            }
        }
        if (prims.empty())
            return VG_OK;
        for (int k = 0; k < 3; ++k)
        {
            if (!std::isfinite(lo[k]) || !std::isfinite(hi[k]) || hi[k] - lo[k] > 1e6)
                return VG_OK;  // no usable box: queries go without the field
        }
        constexpr double kWiden = 0.1, kMinCell = 0.02;
        constexpr int kMaxDim = 200;
        FieldGeom g{};
        double span = 0.0;
        for (int k = 0; k < 3; ++k)
        {
            g.lo[k] = lo[k] - kWiden;
            span = std::max(span, hi[k] + kWiden - g.lo[k]);
        }
        g.cell = std::max(kMinCell, span / kMaxDim);
        for (int k = 0; k < 3; ++k)
            g.dim[k] = std::max(1, static_cast<int>(std::ceil((hi[k] + kWiden - g.lo[k]) / g.cell)));
        const long long cells = static_cast<long long>(g.dim[0]) * g.dim[1] * g.dim[2];
        FieldPrim *d_prims = nullptr;
        VG_CUDA(cudaMalloc(&d_prims, prims.size() * sizeof(FieldPrim)), "cudaMalloc(field primitives)");
        cudaError_t err = cudaMemcpy(d_prims, prims.data(), prims.size() * sizeof(FieldPrim), cudaMemcpyHostToDevice);
        if (err == cudaSuccess)
            err = cudaMalloc(&out.data, cells * sizeof(float));
        if (err == cudaSuccess)
        {
            field_kernel<<<static_cast<unsigned>((cells + 127) / 128), 128>>>(d_prims, static_cast<int>(prims.size()), g,
                                                                             out.data);
            err = cudaGetLastError();
        }
        if (err == cudaSuccess)
            err = cudaDeviceSynchronize();
        cudaFree(d_prims);
        if (err != cudaSuccess)
        {
            out.release();
            return cuda_fail(err, "clearance field");
        }
        for (int k = 0; k < 3; ++k)
        {
            // the grid's corner and the primitives' box, rounded outwards to FP32
            out.g_lo[k] = static_cast<float>(g.lo[k]);
            out.dim[k] = g.dim[k];
            out.p_lo[k] = std::nextafter(static_cast<float>(lo[k]), -INFINITY);
            out.p_hi[k] = std::nextafter(static_cast<float>(hi[k]), INFINITY);
        }
        out.inv_cell = static_cast<float>(1.0 / g.cell);
        out.cell = static_cast<float>(g.cell);
        return VG_OK;
    }
}  // namespace vg
