// Minimal .npy (format 1.0) writer for the dump harness.
#pragma once
#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

namespace npy {

template <typename T> inline const char* descr();
template <> inline const char* descr<double>() { return "<f8"; }
template <> inline const char* descr<float>() { return "<f4"; }
template <> inline const char* descr<int32_t>() { return "<i4"; }
template <> inline const char* descr<uint32_t>() { return "<u4"; }
template <> inline const char* descr<int64_t>() { return "<i8"; }
template <> inline const char* descr<uint8_t>() { return "|u1"; }

template <typename T>
inline void save(const std::string& path, const T* data, const std::vector<size_t>& shape)
{
    std::string sh = "(";
    size_t n = 1;
    for (size_t i = 0; i < shape.size(); i++) {
        sh += std::to_string(shape[i]);
        sh += (shape.size() == 1 || i + 1 < shape.size()) ? "," : "";
        n *= shape[i];
    }
    sh += ")";
    std::string header = std::string("{'descr': '") + descr<T>() +
                         "', 'fortran_order': False, 'shape': " + sh + ", }";
    size_t total = 10 + header.size() + 1;
    size_t pad = (64 - total % 64) % 64;
    header.append(pad, ' ');
    header += '\n';
    FILE* f = std::fopen(path.c_str(), "wb");
    if (!f) { std::perror(path.c_str()); std::exit(3); }
    const unsigned char magic[8] = {0x93, 'N', 'U', 'M', 'P', 'Y', 1, 0};
    std::fwrite(magic, 1, 8, f);
    uint16_t hl = (uint16_t)header.size();
    std::fwrite(&hl, 2, 1, f);
    std::fwrite(header.data(), 1, header.size(), f);
    if (n) std::fwrite(data, sizeof(T), n, f);
    std::fclose(f);
}

template <typename T>
inline void save(const std::string& path, const std::vector<T>& v)
{
    save(path, v.data(), {v.size()});
}

} // namespace npy
