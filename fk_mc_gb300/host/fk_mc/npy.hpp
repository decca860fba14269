// npy.hpp — the NumPy .npy array format (version 1.0): a 10-byte preamble
// (magic "\x93NUMPY", version 1 0, little-endian header length), a Python
// dict literal header ('descr', 'fortran_order', 'shape') padded with spaces
// to a multiple of 64 bytes and ended by '\n', then the raw data in C order.
// The output side of this adapter stores each dataset the reference writes to
// HDF5 as one .npy file (HDF5 is not a dependency here); the graph-lattice
// loader reads its datasets from .npy files the same way.
#pragma once

#include <cstdint>
#include <cstring>
#include <fstream>
#include <stdexcept>
#include <string>
#include <vector>

namespace fk {
namespace npy {

inline bool host_is_little_endian() {
    const std::uint16_t x = 1;
    unsigned char c;
    std::memcpy(&c, &x, 1);
    return c == 1;
}

inline void write_raw(const std::string& path, const char* descr, const void* data, std::size_t bytes,
                      const std::vector<std::size_t>& shape) {
    if (!host_is_little_endian()) throw std::logic_error("npy writer expects a little-endian host");
    std::string shp = "(";
    for (std::size_t i = 0; i < shape.size(); ++i) shp += std::to_string(shape[i]) + (shape.size() == 1 ? "," : (i + 1 < shape.size() ? ", " : ""));
    shp += ")";
    std::string header = std::string("{'descr': '") + descr + "', 'fortran_order': False, 'shape': " + shp + ", }";
    const std::size_t total = 10 + header.size() + 1;
    header.append((64 - total % 64) % 64, ' ');
    header += '\n';
    std::ofstream out(path, std::ios::binary);
    if (!out) throw std::runtime_error("cannot write " + path);
    const unsigned char pre[8] = {0x93, 'N', 'U', 'M', 'P', 'Y', 1, 0};
    out.write(reinterpret_cast<const char*>(pre), 8);
    const std::uint16_t hl = (std::uint16_t)header.size();
    out.write(reinterpret_cast<const char*>(&hl), 2);
    out.write(header.data(), (std::streamsize)header.size());
    if (bytes) out.write(reinterpret_cast<const char*>(data), (std::streamsize)bytes);
    if (!out) throw std::runtime_error("write failed: " + path);
}

inline void write(const std::string& path, const std::vector<double>& v) {
    write_raw(path, "<f8", v.data(), v.size() * sizeof(double), {v.size()});
}

inline void write(const std::string& path, const std::vector<double>& v, std::size_t rows, std::size_t cols) {
    if (rows * cols != v.size()) throw std::logic_error("npy shape does not match the data: " + path);
    write_raw(path, "<f8", v.data(), v.size() * sizeof(double), {rows, cols});
}

// rows of equal length -> one 2-D array
inline void write(const std::string& path, const std::vector<std::vector<double>>& m) {
    const std::size_t rows = m.size(), cols = rows ? m[0].size() : 0;
    std::vector<double> flat;
    flat.reserve(rows * cols);
    for (const auto& r : m) {
        if (r.size() != cols) throw std::logic_error("ragged rows for " + path);
        flat.insert(flat.end(), r.begin(), r.end());
    }
    write(path, flat, rows, cols);
}

// A loaded array: its shape and its values converted to double (real part
// for complex data; `imag` keeps the imaginary parts, empty for real data).
struct array {
    std::vector<std::size_t> shape;
    std::vector<double> data, imag;
    std::size_t size() const { return data.size(); }
};

inline array read(const std::string& path) {
    if (!host_is_little_endian()) throw std::logic_error("npy reader expects a little-endian host");
    std::ifstream in(path, std::ios::binary);
    if (!in) throw std::runtime_error("cannot open " + path);
    unsigned char pre[8];
    in.read(reinterpret_cast<char*>(pre), 8);
    if (!in || pre[0] != 0x93 || std::memcmp(pre + 1, "NUMPY", 5) != 0) throw std::runtime_error("not an npy file: " + path);
    std::size_t hl = 0;
    if (pre[6] == 1) {
        unsigned char b[2];
        in.read(reinterpret_cast<char*>(b), 2);
        hl = b[0] | (b[1] << 8);
    } else if (pre[6] == 2 || pre[6] == 3) {
        unsigned char b[4];
        in.read(reinterpret_cast<char*>(b), 4);
        hl = b[0] | (b[1] << 8) | (b[2] << 16) | ((std::size_t)b[3] << 24);
    } else {
        throw std::runtime_error("unsupported npy version in " + path);
    }
    std::string header(hl, '\0');
    in.read(&header[0], (std::streamsize)hl);
    if (!in) throw std::runtime_error("truncated npy header: " + path);
    auto field = [&](const char* key) -> std::string {
        const std::size_t k = header.find(std::string("'") + key + "'");
        if (k == std::string::npos) throw std::runtime_error(std::string("npy header without ") + key + ": " + path);
        return header.substr(header.find(':', k) + 1);
    };
    std::string descr = field("descr");
    descr = descr.substr(descr.find('\'') + 1);
    descr = descr.substr(0, descr.find('\''));
    const std::string fo = field("fortran_order");
    if (fo.compare(fo.find_first_not_of(' '), 4, "True") == 0)
        throw std::runtime_error("Fortran-order npy not supported: " + path);
    std::string shp = field("shape");
    shp = shp.substr(shp.find('(') + 1, shp.find(')') - shp.find('(') - 1);
    array a;
    std::size_t count = 1, pos = 0;
    while (pos < shp.size()) {
        while (pos < shp.size() && (shp[pos] == ' ' || shp[pos] == ',')) ++pos;
        if (pos >= shp.size()) break;
        std::size_t end = pos;
        while (end < shp.size() && shp[end] >= '0' && shp[end] <= '9') ++end;
        if (end == pos) throw std::runtime_error("bad npy shape in " + path);
        a.shape.push_back(std::stoul(shp.substr(pos, end - pos)));
        count *= a.shape.back();
        pos = end;
    }
    if (descr.size() < 3 || (descr[0] != '<' && descr[0] != '|' && descr[0] != '='))
        throw std::runtime_error("unsupported npy dtype '" + descr + "' in " + path);
    const char kind = descr[1];
    const int width = std::stoi(descr.substr(2));
    std::vector<char> raw(count * (std::size_t)width);
    in.read(raw.data(), (std::streamsize)raw.size());
    if (!in) throw std::runtime_error("truncated npy data: " + path);
    a.data.resize(count);
    for (std::size_t i = 0; i < count; ++i) {
        const char* p = raw.data() + i * width;
        if (kind == 'f' && width == 8) { double v; std::memcpy(&v, p, 8); a.data[i] = v; }
        else if (kind == 'f' && width == 4) { float v; std::memcpy(&v, p, 4); a.data[i] = v; }
        else if (kind == 'i' && width == 8) { std::int64_t v; std::memcpy(&v, p, 8); a.data[i] = (double)v; }
        else if (kind == 'i' && width == 4) { std::int32_t v; std::memcpy(&v, p, 4); a.data[i] = (double)v; }
        else if (kind == 'c' && width == 16) {
            double re, im;
            std::memcpy(&re, p, 8);
            std::memcpy(&im, p + 8, 8);
            if (a.imag.empty()) a.imag.assign(count, 0.0);
            a.data[i] = re;
            a.imag[i] = im;
        } else throw std::runtime_error("unsupported npy dtype '" + descr + "' in " + path);
    }
    return a;
}

}  // namespace npy
}  // namespace fk
