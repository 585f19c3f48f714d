#pragma once

// File formats of the slice example: a reader for the vertex and face lines of Wavefront OBJ, and a writer of
// 8-bit RGB PNG images (zlib stream of stored deflate blocks: no compression, no dependency).
//
// OBJ, as the reference's example reads it (examples/main.cc:52-94 of the antipodal project): `v x y z` adds a
// vertex; `f a b c ...` adds a polygon, fan-triangulated from its first corner; a corner token is `i`, `i/t`,
// `i//n` or `i/t/n`, of which only `i` is used, 1-based, or negative for relative to the vertices read so far.
// Every other line is ignored.  Unlike the reference, an index that is 0 or outside the vertices is an error.

#include <algorithm>
#include <array>
#include <cerrno>
#include <cstddef>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

namespace slice_io
{
struct ObjMesh
{
    std::vector<double> xyz;  // 3 per vertex
    std::vector<int> indices; // 3 per triangle
};

namespace detail
{
inline char const* skip_space(char const* s)
{
    while (*s == ' ' || *s == '\t' || *s == '\r')
        ++s;
    return s;
}
} // namespace detail

// Reads path into mesh; on failure returns false and sets err.
inline bool read_obj(std::string const& path, ObjMesh& mesh, std::string& err)
{
    std::FILE* f = std::fopen(path.c_str(), "rb");
    if (!f)
    {
        err = "could not open '" + path + "'";
        return false;
    }
    std::string line;
    std::vector<int> face;
    long line_no = 0;
    bool ok = true;
    for (int c = 0; ok && c != EOF;)
    {
        line.clear();
        while ((c = std::fgetc(f)) != EOF && c != '\n')
            line.push_back(char(c));
        ++line_no;
        char const* s = detail::skip_space(line.c_str());
        bool const is_v = s[0] == 'v' && (s[1] == ' ' || s[1] == '\t');
        bool const is_f = s[0] == 'f' && (s[1] == ' ' || s[1] == '\t');
        if (is_v)
        {
            s += 1;
            for (int k = 0; k < 3; ++k)
            {
                char* end = nullptr;
                double const x = std::strtod(s, &end);
                if (end == s)
                {
                    err = "line " + std::to_string(line_no) + ": a vertex needs three coordinates";
                    ok = false;
                    break;
                }
                mesh.xyz.push_back(x);
                s = end;
            }
        }
        else if (is_f)
        {
            face.clear();
            s = detail::skip_space(s + 1);
            long const n_vert = long(mesh.xyz.size() / 3);
            while (*s)
            {
                char* end = nullptr;
                errno = 0;
                long const i = std::strtol(s, &end, 10);
                if (end == s || errno != 0)
                {
                    err = "line " + std::to_string(line_no) + ": bad face corner";
                    ok = false;
                    break;
                }
                long const v = i > 0 ? i - 1 : n_vert + i;
                if (i == 0 || v < 0 || v >= n_vert)
                {
                    err = "line " + std::to_string(line_no) + ": vertex index " + std::to_string(i) + " out of range";
                    ok = false;
                    break;
                }
                face.push_back(int(v));
                s = end;
                while (*s && *s != ' ' && *s != '\t' && *s != '\r') // texture / normal indices
                    ++s;
                s = detail::skip_space(s);
            }
            for (std::size_t k = 2; ok && k < face.size(); ++k)
            {
                mesh.indices.push_back(face[0]);
                mesh.indices.push_back(face[k - 1]);
                mesh.indices.push_back(face[k]);
            }
        }
    }
    std::fclose(f);
    return ok;
}

namespace detail
{
inline std::uint32_t crc32(std::uint8_t const* p, std::size_t n, std::uint32_t crc = 0)
{
    // reflected CRC-32 (polynomial 0xEDB88320), the checksum of PNG chunks
    static std::array<std::uint32_t, 256> const table = []
    {
        std::array<std::uint32_t, 256> t{};
        for (std::uint32_t i = 0; i < 256; ++i)
        {
            std::uint32_t c = i;
            for (int k = 0; k < 8; ++k)
                c = (c & 1u) ? 0xEDB88320u ^ (c >> 1) : c >> 1;
            t[i] = c;
        }
        return t;
    }();
    crc = ~crc;
    for (std::size_t i = 0; i < n; ++i)
        crc = table[(crc ^ p[i]) & 0xffu] ^ (crc >> 8);
    return ~crc;
}

inline void put_be32(std::vector<std::uint8_t>& o, std::uint32_t v)
{
    o.push_back(std::uint8_t(v >> 24));
    o.push_back(std::uint8_t(v >> 16));
    o.push_back(std::uint8_t(v >> 8));
    o.push_back(std::uint8_t(v));
}

inline void put_chunk(std::vector<std::uint8_t>& o, char const* type, std::vector<std::uint8_t> const& data)
{
    put_be32(o, std::uint32_t(data.size()));
    std::size_t const start = o.size();
    o.insert(o.end(), type, type + 4);
    o.insert(o.end(), data.begin(), data.end());
    put_be32(o, crc32(o.data() + start, o.size() - start));
}
} // namespace detail

// Writes a width x height RGB image (rows top to bottom, 3 bytes per pixel) as a PNG file.
inline bool write_png(std::string const& path, int width, int height, std::vector<std::uint8_t> const& rgb)
{
    if (width <= 0 || height <= 0 || rgb.size() != std::size_t(width) * height * 3)
        return false;
    std::vector<std::uint8_t> out = {0x89, 'P', 'N', 'G', '\r', '\n', 0x1a, '\n'};
    std::vector<std::uint8_t> ihdr;
    detail::put_be32(ihdr, std::uint32_t(width));
    detail::put_be32(ihdr, std::uint32_t(height));
    ihdr.insert(ihdr.end(), {8, 2, 0, 0, 0}); // 8-bit, RGB, deflate, adaptive filters, no interlace
    detail::put_chunk(out, "IHDR", ihdr);
    // scanlines with filter type 0, in a zlib stream of stored blocks
    std::vector<std::uint8_t> raw;
    raw.reserve((std::size_t(width) * 3 + 1) * height);
    for (int y = 0; y < height; ++y)
    {
        raw.push_back(0);
        auto const* row = rgb.data() + std::size_t(y) * width * 3;
        raw.insert(raw.end(), row, row + std::size_t(width) * 3);
    }
    std::vector<std::uint8_t> z = {0x78, 0x01};
    std::size_t pos = 0;
    do
    {
        std::size_t const len = std::min<std::size_t>(65535, raw.size() - pos);
        bool const last = pos + len == raw.size();
        z.push_back(last ? 1 : 0);
        z.push_back(std::uint8_t(len));
        z.push_back(std::uint8_t(len >> 8));
        z.push_back(std::uint8_t(~len));
        z.push_back(std::uint8_t(~len >> 8));
        z.insert(z.end(), raw.begin() + std::ptrdiff_t(pos), raw.begin() + std::ptrdiff_t(pos + len));
        pos += len;
    } while (pos < raw.size());
    std::uint32_t a = 1, b = 0; // Adler-32 of the uncompressed data
    for (std::uint8_t c : raw)
    {
        a = (a + c) % 65521u;
        b = (b + a) % 65521u;
    }
    detail::put_be32(z, (b << 16) | a);
    detail::put_chunk(out, "IDAT", z);
    detail::put_chunk(out, "IEND", {});
    std::FILE* f = std::fopen(path.c_str(), "wb");
    if (!f)
        return false;
    bool const ok = std::fwrite(out.data(), 1, out.size(), f) == out.size();
    return std::fclose(f) == 0 && ok;
}
} // namespace slice_io
