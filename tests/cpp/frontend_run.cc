// Runs the C++ front end (include/antipodal/cuda/gwn_cuda.hh) the way a reference user would: the +Y-open unit
// cube of the reference tests, a 12^3 grid of queries, eval_gwnr_mesh_batch{,_fractional,_integer} through
// CudaDispatcher / CudaIntersector in both precisions, eval_gwnr_mesh_batch_robust through CudaRobustMeshGwn
// (exact_float), eval_gwnr_parametric_batch_fractional over the open cube's boundary as straight cubic Bezier
// curves (tol 1e-6), and eval_gwnr_parametric_batch{_integer,} with the open cube's five faces as flat bicubic
// patches (CudaBezierPatchIntersector).  Prints one line per query:
//   x y z full_exact full_mixed frac_exact count robust param_frac patch_count param_full
// or "error <status> <message>" when the library throws (e.g. no GPU).
#include <antipodal/math/common.hh>
#include <antipodal/cuda/gwn_cuda.hh>

#include <array>
#include <cstdio>
#include <vector>

int main()
{
    using namespace antipodal;
    std::vector<dvec3> const verts = {{-0.5, -0.5, -0.5}, {0.5, -0.5, -0.5}, {-0.5, 0.5, -0.5}, {0.5, 0.5, -0.5},
                                      {-0.5, -0.5, 0.5},  {0.5, -0.5, 0.5},  {-0.5, 0.5, 0.5},  {0.5, 0.5, 0.5}};
    std::vector<int> const idx = {0, 2, 1, 1, 2, 3, 4, 5, 6, 6, 5, 7, 0, 4, 2, 2, 4, 6, 1, 3, 5, 5, 3, 7, 0, 1, 4, 4, 1, 5};
    std::vector<weighted_dsegment3> const bnd = {
        {{verts[6], verts[2]}, 1.0}, {{verts[7], verts[6]}, 1.0}, {{verts[3], verts[7]}, 1.0}, {{verts[2], verts[3]}, 1.0}};
    dvec3 const x0 = normalize(dvec3{0.31, 0.57, 0.76});
    std::vector<dvec3> pts;
    int const n = 12;
    for (int k = 0; k < n; ++k)
        for (int j = 0; j < n; ++j)
            for (int i = 0; i < n; ++i)
                pts.push_back({-1.5 + 3.0 * (i + 0.37) / n, -1.5 + 3.0 * (j + 0.61) / n, -1.5 + 3.0 * (k + 0.19) / n});
    std::span<dvec3 const> const P{pts};
    std::span<weighted_dsegment3 const> const B{bnd};
    try
    {
        cuda::CudaDispatcher disp;
        cuda::CudaIntersector<double> const isect{disp, verts, idx};
        std::vector<double> exact(pts.size()), mixed(pts.size()), frac(pts.size());
        std::vector<int> counts(pts.size());
        eval_gwnr_mesh_batch(disp, isect, P, std::span<double>{exact}, x0, B);
        eval_gwnr_mesh_batch_fractional(disp, P, std::span<double>{frac}, x0, B);
        eval_gwnr_mesh_batch_integer(disp, isect, P, std::span<int>{counts}, x0);
        disp.set_precision(cuda::precision::mixed);
        eval_gwnr_mesh_batch(disp, isect, P, std::span<double>{mixed}, x0, B);
        disp.set_precision(cuda::precision::exact);

        std::vector<double> robust(pts.size()), param(pts.size());
        cuda::CudaRobustMeshGwn<double> const rob{disp, verts, idx, B};
        eval_gwnr_mesh_batch_robust(disp, rob, P, std::span<double>{robust});

        std::vector<std::array<dvec3, 4>> curves;
        for (auto const& ws : bnd)
        {
            dvec3 const a = ws.segment.pos0, b = ws.segment.pos1;
            curves.push_back({a, dvec3{(2 * a.x + b.x) / 3, (2 * a.y + b.y) / 3, (2 * a.z + b.z) / 3},
                              dvec3{(a.x + 2 * b.x) / 3, (a.y + 2 * b.y) / 3, (a.z + 2 * b.z) / 3}, b});
        }
        integrate_config cfg;
        cfg.tol = 1e-6;
        eval_gwnr_parametric_batch_fractional(disp, P, std::span<double>{param}, x0,
                                              cuda::CubicBezierBoundary{std::span<std::array<dvec3, 4> const>{curves}},
                                              cfg);
        // each face as a flat bicubic patch: P[i][j] = a + (j/3)(b - a) + (i/3)(c - a) for the face's first triangle
        // (a, b, c), so that S_u x S_v is that triangle's normal
        std::vector<std::array<dvec3, 16>> patches;
        for (size_t f = 0; f < idx.size() / 6; ++f)
        {
            dvec3 const a = verts[idx[6 * f]], b = verts[idx[6 * f + 1]], c = verts[idx[6 * f + 2]];
            std::array<dvec3, 16> g{};
            for (int i = 0; i < 4; ++i)
                for (int j = 0; j < 4; ++j)
                    g[4 * i + j] = dvec3{a.x + j * (b.x - a.x) / 3 + i * (c.x - a.x) / 3,
                                         a.y + j * (b.y - a.y) / 3 + i * (c.y - a.y) / 3,
                                         a.z + j * (b.z - a.z) / 3 + i * (c.z - a.z) / 3};
            patches.push_back(g);
        }
        cuda::CudaBezierPatchIntersector const pint{disp, std::span<std::array<dvec3, 16> const>{patches}};
        std::vector<int> pcount(pts.size());
        std::vector<double> pfull(pts.size());
        eval_gwnr_parametric_batch_integer(disp, pint, P, std::span<int>{pcount}, x0);
        eval_gwnr_parametric_batch(disp, pint, P, std::span<double>{pfull}, x0,
                                   cuda::CubicBezierBoundary{std::span<std::array<dvec3, 4> const>{curves}}, cfg);
        for (size_t q = 0; q < pts.size(); ++q)
            std::printf("%.17g %.17g %.17g %.17g %.17g %.17g %d %.17g %.17g %d %.17g\n", pts[q].x, pts[q].y, pts[q].z,
                        exact[q], mixed[q], frac[q], counts[q], robust[q], param[q], pcount[q], pfull[q]);
    }
    catch (cuda::Error const& e)
    {
        std::printf("error %d %s\n", e.status(), e.what());
        return 3;
    }
    return 0;
}
