// NPY v1.0 writer with the on-disk format of the reference's
// simulations/save_npy.cpp:34-75 (and save_npy.hpp:91-145): magic
// "\x93NUMPY", version 1.0, a little-endian uint16 header length, and a
// header dict "{'descr': '<f8', 'fortran_order': True, 'shape': (n0, n1, n2, ), }"
// padded with spaces and a final '\n' so that the data starts on a 64-byte
// boundary.  layout_left arrays are written as fortran_order True, in memory
// order.  Unlike the reference driver, callers pass host memory (copy device
// data out first), so the writer never dereferences device pointers.
#pragma once

#include <bit>
#include <cstddef>
#include <cstdint>
#include <fstream>
#include <ostream>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>

namespace euler_npy {

template <class T>
std::string descr()
{
    static_assert(std::is_floating_point_v<T> || std::is_integral_v<T>, "unsupported element type");
    char const order = sizeof(T) == 1 ? '|' : (std::endian::native == std::endian::little ? '<' : '>');
    char const kind = std::is_floating_point_v<T> ? 'f' : (std::is_signed_v<T> ? 'i' : 'u');
    return std::string(1, order) + kind + std::to_string(sizeof(T));
}

inline std::string header(std::string const& descr, bool fortran_order, std::vector<std::size_t> const& shape)
{
    std::string shape_str = "(";
    for (std::size_t e : shape) {
        shape_str += std::to_string(e) + ", ";
    }
    shape_str += ")";
    std::string h = "{'descr': '" + descr + "', 'fortran_order': " + (fortran_order ? "True" : "False") +
                    ", 'shape': " + shape_str + ", }";
    std::size_t const prefix = 6 + 2 + 2; // magic, version, header length
    std::size_t const used = prefix + h.size() + 1;
    h += std::string(((used + 63) / 64) * 64 - used, ' ');
    h += '\n';
    if (h.size() > 0xffff) {
        throw std::runtime_error("npy header too large for format 1.0");
    }
    return h;
}

template <class T>
void write(std::ostream& os, T const* data, std::vector<std::size_t> const& shape, bool fortran_order)
{
    std::string const h = header(descr<T>(), fortran_order, shape);
    auto const hlen = static_cast<std::uint16_t>(h.size());
    unsigned char const pre[10] = {0x93, 'N', 'U', 'M', 'P', 'Y', 1, 0,
                                   static_cast<unsigned char>(hlen & 0xff), static_cast<unsigned char>(hlen >> 8)};
    os.write(reinterpret_cast<char const*>(pre), sizeof(pre));
    os.write(h.data(), static_cast<std::streamsize>(h.size()));
    std::size_t n = 1;
    for (std::size_t e : shape) {
        n *= e;
    }
    os.write(reinterpret_cast<char const*>(data), static_cast<std::streamsize>(n * sizeof(T)));
}

template <class T>
void write_file(std::string const& path, T const* data, std::vector<std::size_t> const& shape, bool fortran_order)
{
    std::ofstream f(path, std::ios::binary);
    if (!f) {
        throw std::runtime_error("cannot open " + path);
    }
    f.exceptions(std::ios::failbit | std::ios::badbit);
    write(f, data, shape, fortran_order);
}

} // namespace euler_npy
