// RREATBL v1 container reader: a 64-byte little-endian prefix, a JSON header
// whose values are all strings, and one deflate payload holding byte-plane
// shuffled columns in header order.  The format is the reference's table
// bundle format (native_amrex_rrea/include/rrea/RreaTableContainer.H:1-17);
// this reader is written from that layout description.
#pragma once

#include "json_lite.hpp"

#include <zlib.h>

#include <cmath>
#include <cstdint>
#include <cstring>
#include <fstream>
#include <iterator>
#include <stdexcept>
#include <string>
#include <vector>

namespace rrea_host {

struct RreaTableContainer {
    JsonValue header;
    std::string payload;  // inflated, still byte-plane shuffled per column
    std::string path;

    std::vector<std::string> list(std::string const& key) const
    {
        std::vector<std::string> out;
        std::string const text = header.str(key);
        std::size_t start = 0;
        while (start <= text.size()) {
            std::size_t const stop = text.find(',', start);
            std::string item = text.substr(start, stop == std::string::npos ? std::string::npos : stop - start);
            // trim blanks
            std::size_t a = item.find_first_not_of(" \t");
            std::size_t b = item.find_last_not_of(" \t");
            out.push_back(a == std::string::npos ? std::string() : item.substr(a, b - a + 1));
            if (stop == std::string::npos) {
                break;
            }
            start = stop + 1;
        }
        return out;
    }

    std::size_t rows() const { return static_cast<std::size_t>(std::stoull(header.str("rows"))); }

    bool find_column(std::string const& name, std::size_t& offset,
                     std::size_t& length, std::string& dtype) const
    {
        auto const names = list("column_names");
        auto const dtypes = list("column_dtypes");
        auto const sizes = list("column_bytes");
        if (names.size() != dtypes.size() || names.size() != sizes.size()) {
            throw std::runtime_error("RREATBL: column lists disagree in " + path);
        }
        offset = 0;
        for (std::size_t i = 0; i < names.size(); ++i) {
            std::size_t const bytes = static_cast<std::size_t>(std::stoull(sizes[i]));
            if (names[i] == name) {
                length = bytes;
                dtype = dtypes[i];
                if (offset + length > payload.size()) {
                    throw std::runtime_error("RREATBL: column past payload: " + name);
                }
                return true;
            }
            offset += bytes;
        }
        return false;
    }

    static std::size_t item_bytes(std::string const& dtype)
    {
        if (dtype == "f8") return 8;
        if (dtype == "i4" || dtype == "u4") return 4;
        if (dtype == "u2") return 2;
        if (dtype == "u1") return 1;
        if (dtype == "str") return 0;
        throw std::runtime_error("RREATBL: unsupported dtype " + dtype);
    }

    // Numeric column decoded to double, in row order.
    std::vector<double> column(std::string const& name) const
    {
        std::size_t offset = 0, length = 0;
        std::string dtype;
        if (!find_column(name, offset, length, dtype)) {
            throw std::runtime_error("RREATBL: " + path + " has no column " + name);
        }
        std::size_t const width = item_bytes(dtype);
        if (width == 0) {
            throw std::runtime_error("RREATBL: column " + name + " is text");
        }
        std::size_t const count = length / width;
        std::vector<unsigned char> plain(length);
        unsigned char const* planes =
            reinterpret_cast<unsigned char const*>(payload.data()) + offset;
        for (std::size_t k = 0; k < width; ++k) {
            for (std::size_t i = 0; i < count; ++i) {
                plain[i * width + k] = planes[k * count + i];
            }
        }
        std::vector<double> values(count);
        for (std::size_t i = 0; i < count; ++i) {
            unsigned char const* item = plain.data() + i * width;
            if (dtype == "f8") {
                double d;
                std::memcpy(&d, item, 8);
                if (!std::isfinite(d)) {
                    throw std::runtime_error("RREATBL: non-finite value in " + name);
                }
                values[i] = d;
            } else if (dtype == "i4") {
                std::int32_t v;
                std::memcpy(&v, item, 4);
                values[i] = static_cast<double>(v);
            } else {
                std::uint64_t v = 0;
                for (std::size_t b = 0; b < width; ++b) {
                    v |= static_cast<std::uint64_t>(item[b]) << (8 * b);
                }
                values[i] = static_cast<double>(v);
            }
        }
        return values;
    }

    std::vector<std::string> text_column(std::string const& name) const
    {
        std::size_t offset = 0, length = 0;
        std::string dtype;
        if (!find_column(name, offset, length, dtype) || dtype != "str") {
            throw std::runtime_error("RREATBL: no text column " + name);
        }
        std::vector<std::string> out;
        std::string const blob = payload.substr(offset, length);
        std::size_t start = 0;
        while (start <= blob.size()) {
            std::size_t const stop = blob.find('\n', start);
            out.push_back(blob.substr(start, stop == std::string::npos ? std::string::npos : stop - start));
            if (stop == std::string::npos) break;
            start = stop + 1;
        }
        return out;
    }
};

inline std::uint64_t rreatbl_read_le(std::string const& b, std::size_t off, std::size_t w)
{
    std::uint64_t v = 0;
    for (std::size_t i = 0; i < w; ++i) {
        v |= static_cast<std::uint64_t>(static_cast<unsigned char>(b[off + i])) << (8 * i);
    }
    return v;
}

inline RreaTableContainer ReadRreaTableContainer(std::string const& path)
{
    std::ifstream in(path, std::ios::binary);
    if (!in) {
        throw std::runtime_error("RREATBL: could not open " + path);
    }
    std::string const bytes((std::istreambuf_iterator<char>(in)), std::istreambuf_iterator<char>());
    if (bytes.size() < 64 || bytes.compare(0, 7, "RREATBL") != 0 || bytes[7] != '\0') {
        throw std::runtime_error("RREATBL: bad magic in " + path);
    }
    if (rreatbl_read_le(bytes, 8, 4) != 1u || rreatbl_read_le(bytes, 12, 4) != 0x01020304u
        || rreatbl_read_le(bytes, 20, 4) != 0u) {
        throw std::runtime_error("RREATBL: incompatible version/endianness in " + path);
    }
    std::size_t const header_bytes = static_cast<std::size_t>(rreatbl_read_le(bytes, 16, 4));
    std::uint64_t const payload_bytes = rreatbl_read_le(bytes, 24, 8);
    if (bytes.size() != 64 + header_bytes + payload_bytes) {
        throw std::runtime_error("RREATBL: size mismatch in " + path);
    }
    RreaTableContainer c;
    c.path = path;
    c.header = ParseJson(bytes.substr(64, header_bytes));
    // The header's column byte counts give the exact inflated size.
    std::size_t inflated = 0;
    for (auto const& s : c.list("column_bytes")) {
        inflated += static_cast<std::size_t>(std::stoull(s));
    }
    c.payload.assign(inflated, '\0');
    uLongf produced = static_cast<uLongf>(inflated);
    int const status = uncompress(
        reinterpret_cast<Bytef*>(&c.payload[0]), &produced,
        reinterpret_cast<Bytef const*>(bytes.data() + 64 + header_bytes),
        static_cast<uLong>(payload_bytes));
    if (status != Z_OK || produced != inflated) {
        throw std::runtime_error("RREATBL: inflate failed for " + path);
    }
    return c;
}

}  // namespace rrea_host
