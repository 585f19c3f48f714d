// Test driver of examples/obj_png.hh: reads the OBJ file argv[1] and prints its vertex count, then one triangle
// per line; writes argv[2] as a width x height PNG of a pattern the test recomputes (r = x, g = y, b = x ^ y, all
// mod 256).  Exit status 2 and the reader's message on stderr when the OBJ file is rejected.
#include "../../examples/obj_png.hh"

#include <cstdio>
#include <cstdlib>

int main(int argc, char** argv)
{
    if (argc < 5)
        return 1;
    slice_io::ObjMesh mesh;
    std::string err;
    if (!slice_io::read_obj(argv[1], mesh, err))
    {
        std::fprintf(stderr, "%s\n", err.c_str());
        return 2;
    }
    std::printf("%zu\n", mesh.xyz.size() / 3);
    for (std::size_t t = 0; t + 2 < mesh.indices.size(); t += 3)
        std::printf("%d %d %d\n", mesh.indices[t], mesh.indices[t + 1], mesh.indices[t + 2]);
    int const w = std::atoi(argv[3]), h = std::atoi(argv[4]);
    std::vector<std::uint8_t> rgb(std::size_t(w) * h * 3);
    for (int y = 0; y < h; ++y)
        for (int x = 0; x < w; ++x)
        {
            std::uint8_t* p = &rgb[(std::size_t(y) * w + x) * 3];
            p[0] = std::uint8_t(x), p[1] = std::uint8_t(y), p[2] = std::uint8_t(x ^ y);
        }
    return slice_io::write_png(argv[2], w, h, rgb) ? 0 : 3;
}
