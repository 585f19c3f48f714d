// The reference's slice example (examples/main.cc of the antipodal project) on the GPU: load an OBJ triangle
// mesh, evaluate its generalized winding number on a square grid over a plane, write the slice as a PNG.  The
// command line and the image are the reference's; the evaluation runs through this library's C++ front end
// (CudaDispatcher, CudaIntersector, the device boundary extraction and eval_gwnr_mesh_batch) instead of
// PoolDispatcher and NaiveIntersector, with the same values: counts bit for bit, the fractional term in the
// reference's FP64 arithmetic (or, with the precision argument "mixed", within 1e-7).
//
//   slice <input.obj> <output.png> <resolution> [slice_pos=0.5] [nx ny nz = 0 1 0] [extent=1.2]
//         [precision=exact|mixed] [values.bin]
//
// slice_pos places the plane along its normal between the mesh's extremes (0 and 1); extent is the side of the
// square window relative to the mesh's larger extent in the plane.  values.bin, if given, receives the queries and
// their winding numbers as resolution^2 rows of four doubles (x, y, z, w), rows of the grid bottom to top.
//
// Build (the reference's headers, or any header with the same value types, on the include path):
//   g++ -std=c++20 -O2 -I include -I <antipodal>/src examples/slice.cc -o slice
//       -L antipodal_gb300 -lantipodal_gb300 -Wl,-rpath,antipodal_gb300

#include <antipodal/cuda/gwn_cuda.hh>

#include "obj_png.hh"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <limits>
#include <string>
#include <vector>

namespace
{
using V = antipodal::vec3<double>;

V scale(double s, V a)
{
    return {s * a.x, s * a.y, s * a.z};
}
V add(V a, V b)
{
    return {a.x + b.x, a.y + b.y, a.z + b.z};
}
double dot(V a, V b)
{
    return a.x * b.x + a.y * b.y + a.z * b.z;
}
V cross(V a, V b)
{
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
V unit(V a)
{
    double const n = std::sqrt(dot(a, a));
    return {a.x / n, a.y / n, a.z / n};
}

// The reference's diverging colour map: w clamped to [-1, 1] blends from #2F5994 (w = 0, outside) towards
// #F3E676 (w = 1, inside) or #D2552E (w = -1).
void colour(double w, std::uint8_t* px)
{
    static constexpr double outside[3] = {47, 89, 148}, inside[3] = {243, 230, 118}, negative[3] = {210, 85, 46};
    w = std::clamp(w, -1.0, 1.0);
    double const* to = w >= 0 ? inside : negative;
    double const t = std::fabs(w);
    for (int c = 0; c < 3; ++c)
        px[c] = std::uint8_t(std::lround(std::clamp(outside[c] + (to[c] - outside[c]) * t, 0.0, 255.0)));
}

double seconds_since(std::chrono::steady_clock::time_point t0)
{
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}
} // namespace

int main(int argc, char** argv)
{
    if (argc < 4)
    {
        std::fprintf(stderr,
                     "usage: %s <input.obj> <output.png> <resolution> [slice_pos=0.5] [nx ny nz = 0 1 0] "
                     "[extent=1.2] [precision=exact|mixed] [values.bin]\n",
                     argv[0]);
        return 1;
    }
    std::string const obj_path = argv[1], png_path = argv[2];
    int const res = std::atoi(argv[3]);
    double const slice_pos = argc > 4 ? std::atof(argv[4]) : 0.5;
    V const normal = argc > 7 ? V{std::atof(argv[5]), std::atof(argv[6]), std::atof(argv[7])} : V{0, 1, 0};
    double const extent = argc > 8 ? std::atof(argv[8]) : 1.2;
    std::string const prec = argc > 9 ? argv[9] : "exact";
    std::string const dump = argc > 10 ? argv[10] : "";
    if (res <= 0)
    {
        std::fprintf(stderr, "error: resolution must be positive\n");
        return 1;
    }
    if (prec != "exact" && prec != "mixed")
    {
        std::fprintf(stderr, "error: precision must be exact or mixed\n");
        return 1;
    }
    if (!(dot(normal, normal) > 0))
    {
        std::fprintf(stderr, "error: the plane normal must not be zero\n");
        return 1;
    }

    slice_io::ObjMesh mesh;
    std::string err;
    if (!slice_io::read_obj(obj_path, mesh, err))
    {
        std::fprintf(stderr, "error: %s\n", err.c_str());
        return 1;
    }
    if (mesh.xyz.empty() || mesh.indices.empty())
    {
        std::fprintf(stderr, "error: no triangles loaded from '%s'\n", obj_path.c_str());
        return 1;
    }
    std::vector<V> verts(mesh.xyz.size() / 3);
    for (std::size_t i = 0; i < verts.size(); ++i)
        verts[i] = {mesh.xyz[3 * i], mesh.xyz[3 * i + 1], mesh.xyz[3 * i + 2]};
    std::printf("loaded %zu vertices, %zu triangles\n", verts.size(), mesh.indices.size() / 3);

    // the plane's frame (n, u, v) and the window: the same construction as the reference, so the pixels sample
    // the same points
    V const n = unit(normal);
    V const helper = std::fabs(n.x) < 0.9 ? V{1, 0, 0} : V{0, 1, 0};
    V const u = unit(cross(helper, n));
    V const v = cross(n, u);
    double dlo = std::numeric_limits<double>::max(), dhi = std::numeric_limits<double>::lowest();
    double alo = dlo, ahi = dhi, blo = dlo, bhi = dhi;
    for (V const& p : verts)
    {
        double const d = dot(p, n), a = dot(p, u), b = dot(p, v);
        dlo = std::min(dlo, d), dhi = std::max(dhi, d);
        alo = std::min(alo, a), ahi = std::max(ahi, a);
        blo = std::min(blo, b), bhi = std::max(bhi, b);
    }
    V const anchor = scale(dlo + slice_pos * (dhi - dlo), n);
    double const ac = (alo + ahi) / 2, bc = (blo + bhi) / 2;
    double const larger = std::max(ahi - alo, bhi - blo);
    double const side = extent * (larger > 0 ? larger : 1.0);
    std::vector<V> points(std::size_t(res) * res);
    for (int j = 0; j < res; ++j)
    {
        double const bv = bc + ((j + 0.5) / res - 0.5) * side;
        for (int i = 0; i < res; ++i)
        {
            double const au = ac + ((i + 0.5) / res - 0.5) * side;
            points[std::size_t(j) * res + i] = add(add(anchor, scale(au, u)), scale(bv, v));
        }
    }

    std::vector<double> wn(points.size());
    try
    {
        namespace agc = antipodal::cuda;
        auto const t0 = std::chrono::steady_clock::now();
        agc::CudaDispatcher disp(0, nullptr, prec == "mixed" ? agc::precision::mixed : agc::precision::exact);
        std::span<V const> const vs{verts};
        std::span<int const> const is{mesh.indices};
        auto const boundary = antipodal::build_boundary_segments<double>(disp, vs, is);
        agc::CudaIntersector<double> isect{disp, vs, is};
        std::printf("open boundary: %zu segments\n", boundary.size());
        V const x0 = unit(V{0.31, 0.57, 0.76}); // the reference's fixed direction
        auto const t1 = std::chrono::steady_clock::now();
        antipodal::eval_gwnr_mesh_batch(disp, isect, std::span<V const>{points}, std::span<double>{wn}, x0,
                                        std::span<antipodal::weighted_segment3<double> const>{boundary});
        std::printf("setup %.3f ms, %zu queries in %.3f ms (%s)\n", 1e3 * std::chrono::duration<double>(t1 - t0).count(),
                    points.size(), 1e3 * seconds_since(t1), prec.c_str());
    }
    catch (std::exception const& e)
    {
        std::fprintf(stderr, "error: %s\n", e.what());
        return 1;
    }

    // image rows top to bottom: +v up
    std::vector<std::uint8_t> rgb(std::size_t(res) * res * 3);
    for (int j = 0; j < res; ++j)
        for (int i = 0; i < res; ++i)
            colour(wn[std::size_t(res - 1 - j) * res + i], &rgb[(std::size_t(j) * res + i) * 3]);
    if (!slice_io::write_png(png_path, res, res, rgb))
    {
        std::fprintf(stderr, "error: failed to write '%s'\n", png_path.c_str());
        return 1;
    }
    if (!dump.empty())
    {
        std::vector<double> rows;
        rows.reserve(points.size() * 4);
        for (std::size_t k = 0; k < points.size(); ++k)
            rows.insert(rows.end(), {points[k].x, points[k].y, points[k].z, wn[k]});
        std::FILE* f = std::fopen(dump.c_str(), "wb");
        bool const ok = f && std::fwrite(rows.data(), sizeof(double), rows.size(), f) == rows.size();
        if (f)
            std::fclose(f);
        if (!ok)
        {
            std::fprintf(stderr, "error: failed to write '%s'\n", dump.c_str());
            return 1;
        }
    }
    std::printf("wrote %dx%d slice to '%s'\n", res, res, png_path.c_str());
    return 0;
}
