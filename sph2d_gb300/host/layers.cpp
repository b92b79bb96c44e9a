// layers.cpp — particle layer CSV files of an experiment directory.
//
// Format of the reference's dump/data layers (sources/RRSPH_COMMON/src/Output.cpp:80-221):
// header x,y[,z],itype[,vx,vy[,vz]][,rho][,p]; fields separated by ',', rows
// ended by '\n'; doubles printed by std::to_string ("%f"), itype as an integer.
// Reading follows loadArrays (sources/RRSPH_COMMON/src/Input.cpp:203-236):
// columns are looked up by name and the row count must equal ntotal.
#include "../../include/rrsph_cuda.h"
#include "error.hpp"

#include <charconv>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <filesystem>
#include <algorithm>
#include <string>
#include <thread>
#include <vector>

using rrsph::set_error;

namespace {

// std::to_string(double) is specified as printf("%f"): the exact binary value
// rounded to 6 decimals, ties to even. For a finite |v| < 9e12 that is done
// here with integers: v = m * 2^e (e < 0 in that range), and
// q = m * 10^6 / 2^-e rounded half to even in 128-bit arithmetic is the value
// in millionths, printed as q / 10^6 '.' q % 10^6 with six digits. The sign of
// a negative value that rounds to zero (and of -0.0) is kept, as printf keeps
// it. Other values (infinities, NaN, |v| >= 9e12) go to std::to_chars with
// fixed format and precision 6, which is specified to match printf.
// Writes at most kMaxNumberChars characters at o; returns the end.
constexpr size_t kMaxNumberChars = 330;
struct Digits2 {  // "00", "01", ..., "99"
    char d[200];
    constexpr Digits2() : d() {
        for (int i = 0; i < 100; i++) {
            d[2 * i] = (char)('0' + i / 10);
            d[2 * i + 1] = (char)('0' + i % 10);
        }
    }
};
constexpr Digits2 kDigits2{};
char* put_f(char* o, double v) {
    uint64_t bits;
    std::memcpy(&bits, &v, sizeof(bits));
    const int be = (int)((bits >> 52) & 0x7ff);
    const int e = (be ? be : 1) - 1075;
    if (be == 0x7ff || std::fabs(v) >= 9.0e12 || e >= 0) {
        const auto res = std::to_chars(o, o + kMaxNumberChars, v, std::chars_format::fixed, 6);
        if (res.ec == std::errc()) return res.ptr;
        const int n = std::snprintf(o, kMaxNumberChars, "%f", v);
        return o + (n > 0 ? std::min<size_t>((size_t)n, kMaxNumberChars - 1) : 0);
    }
    const uint64_t m = (bits & ((uint64_t(1) << 52) - 1)) | (be ? uint64_t(1) << 52 : 0);
    const int s = -e;  // m * 10^6 < 2^73: from s = 74 on, q = 0 and the remainder is below one half
    uint64_t q = 0;
    if (s < 74) {
        const unsigned __int128 num = (unsigned __int128)m * 1000000u;
        unsigned __int128 qq = num >> s;
        const unsigned __int128 rem = num - (qq << s);
        const unsigned __int128 half = (unsigned __int128)1 << (s - 1);
        if (rem > half || (rem == half && (qq & 1))) qq++;
        q = (uint64_t)qq;
    }
    if (bits >> 63) *o++ = '-';
    uint64_t ip = q / 1000000;  // < 9e12: at most 13 digits
    const uint32_t fp = (uint32_t)(q % 1000000);
    // the integer part, two digits at a time from the right
    char t[16];
    int k = 16;
    while (ip >= 100) {
        k -= 2;
        std::memcpy(t + k, kDigits2.d + 2 * (ip % 100), 2);
        ip /= 100;
    }
    if (ip >= 10) {
        k -= 2;
        std::memcpy(t + k, kDigits2.d + 2 * ip, 2);
    } else {
        t[--k] = (char)('0' + ip);
    }
    std::memcpy(o, t + k, (size_t)(16 - k));
    o += 16 - k;
    *o++ = '.';
    std::memcpy(o, kDigits2.d + 2 * (fp / 10000), 2);
    std::memcpy(o + 2, kDigits2.d + 2 * (fp / 100 % 100), 2);
    std::memcpy(o + 4, kDigits2.d + 2 * (fp % 100), 2);
    return o + 6;
}

}  // namespace

extern "C" int rrsph_layer_time_from_path(const char* path, double* t) {
    if (!path || !t) return set_error(RRSPH_ERR_INVALID_ARGUMENT, "rrsph_layer_time_from_path: null argument");
    const std::string stem = std::filesystem::path(path).stem().string();
    char* end = nullptr;
    const double v = std::strtod(stem.c_str(), &end);
    if (end == stem.c_str()) return set_error(RRSPH_ERR_PARSE, "layer name is not a time: " + stem);
    *t = v;
    return RRSPH_OK;
}

extern "C" int rrsph_layer_read(const char* csv_path, const rrsph_params* p, double* r, uint32_t stride, double* v,
                                double* rho, double* pres, int32_t* itype) {
    if (!csv_path || !p || !r || !v || !rho || !itype)
        return set_error(RRSPH_ERR_INVALID_ARGUMENT, "rrsph_layer_read: null argument");
    if (stride < p->dim) return set_error(RRSPH_ERR_INVALID_ARGUMENT, "rrsph_layer_read: stride < dim");
    FILE* f = std::fopen(csv_path, "rb");
    if (!f) return set_error(RRSPH_ERR_IO, std::string("cannot open layer ") + csv_path);
    std::string data;
    {
        char buf[1 << 16];
        size_t got;
        while ((got = std::fread(buf, 1, sizeof(buf), f)) > 0) data.append(buf, got);
        std::fclose(f);
    }
    // header
    size_t pos = data.find('\n');
    if (pos == std::string::npos) return set_error(RRSPH_ERR_PARSE, "layer has no header line");
    std::vector<std::string> cols;
    {
        std::string h = data.substr(0, pos);
        if (!h.empty() && h.back() == '\r') h.pop_back();
        size_t s = 0;
        for (;;) {
            const size_t e = h.find(',', s);
            std::string name = h.substr(s, e == std::string::npos ? std::string::npos : e - s);
            if (name.size() >= 2 && name.front() == '"' && name.back() == '"') name = name.substr(1, name.size() - 2);
            cols.push_back(name);
            if (e == std::string::npos) break;
            s = e + 1;
        }
    }
    const bool d3 = p->dim == 3;
    auto col = [&](const char* n) -> int {
        for (size_t i = 0; i < cols.size(); i++)
            if (cols[i] == n) return (int)i;
        return -1;
    };
    const int cx = col("x"), cy = col("y"), cz = d3 ? col("z") : -1, ct = col("itype"), cvx = col("vx"),
              cvy = col("vy"), cvz = d3 ? col("vz") : -1, cr = col("rho"), cp = col("p");
    if (cx < 0 || cy < 0 || ct < 0 || cvx < 0 || cvy < 0 || cr < 0 || (d3 && (cz < 0 || cvz < 0)))
        return set_error(RRSPH_ERR_PARSE, std::string("layer ") + csv_path + " lacks a column of x,y,[z],itype,vx,vy,[vz],rho");
    std::vector<const char*> field(cols.size());
    uint64_t row = 0;
    size_t i = pos + 1;
    const size_t n = data.size();
    while (i < n) {
        // split one line in place
        size_t k = 0;
        size_t s = i;
        while (i < n && data[i] != '\n') {
            if (data[i] == ',') {
                if (k < field.size()) field[k++] = data.c_str() + s;
                s = i + 1;
            }
            i++;
        }
        const bool empty_line = (i == s) && k == 0;
        if (k < field.size()) field[k++] = data.c_str() + s;
        i++;  // skip '\n'
        if (empty_line) continue;
        if (k != field.size()) return set_error(RRSPH_ERR_PARSE, "layer row " + std::to_string(row) + " has a wrong number of fields");
        if (row >= p->ntotal) return set_error(RRSPH_ERR_PARSE, "dump corrupted: dump ntotal doesn't match params.ntotal!");
        double* rr = r + row * stride;
        double* vv = v + row * stride;
        rr[0] = std::strtod(field[cx], nullptr);
        rr[1] = std::strtod(field[cy], nullptr);
        if (d3) rr[2] = std::strtod(field[cz], nullptr);
        itype[row] = (int32_t)std::strtol(field[ct], nullptr, 10);
        vv[0] = std::strtod(field[cvx], nullptr);
        vv[1] = std::strtod(field[cvy], nullptr);
        if (d3) vv[2] = std::strtod(field[cvz], nullptr);
        rho[row] = std::strtod(field[cr], nullptr);
        if (pres) pres[row] = cp >= 0 ? std::strtod(field[cp], nullptr) : 0.0;
        row++;
    }
    if (row != p->ntotal) return set_error(RRSPH_ERR_PARSE, "dump corrupted: dump ntotal doesn't match params.ntotal!");
    return RRSPH_OK;
}

extern "C" int rrsph_layer_write(const char* csv_path, const rrsph_params* p, const double* r, uint32_t stride,
                                 const double* v, const double* rho, const double* pres, const int32_t* itype,
                                 int dump) {
    if (!csv_path || !p || !r || !itype) return set_error(RRSPH_ERR_INVALID_ARGUMENT, "rrsph_layer_write: null argument");
    if (stride < p->dim) return set_error(RRSPH_ERR_INVALID_ARGUMENT, "rrsph_layer_write: stride < dim");
    const bool d3 = p->dim == 3;
    const bool wv = dump ? true : (p->save_velocity && v);
    const bool wr = dump ? true : (p->save_density && rho);
    const bool wp = dump ? true : (p->save_pressure && pres);
    if ((wv && !v) || (wr && !rho) || (wp && !pres))
        return set_error(RRSPH_ERR_INVALID_ARGUMENT, "rrsph_layer_write: a dump needs r, itype, v, rho and p");
    std::string head = d3 ? "x,y,z,itype" : "x,y,itype";
    if (wv) head += d3 ? ",vx,vy,vz" : ",vx,vy";
    if (wr) head += ",rho";
    if (wp) head += ",p";
    head += '\n';
    // the lines of particles [i0, i1) into out
    const size_t max_line = 8 * (kMaxNumberChars + 1) + 32;
    auto lines = [&](uint64_t i0, uint64_t i1, std::string& out) {
        out.resize((size_t)(i1 - i0) * 64 + max_line);
        size_t used = 0;
        for (uint64_t i = i0; i < i1; i++) {
            if (out.size() - used < max_line) out.resize(2 * out.size());
            char* const b = &out[0] + used;
            char* o = b;
            const double* ri = r + i * stride;
            o = put_f(o, ri[0]);
            *o++ = ',';
            o = put_f(o, ri[1]);
            *o++ = ',';
            if (d3) {
                o = put_f(o, ri[2]);
                *o++ = ',';
            }
            o = std::to_chars(o, o + 16, (long)itype[i]).ptr;
            if (wv) {
                const double* vi = v + i * stride;
                *o++ = ',';
                o = put_f(o, vi[0]);
                *o++ = ',';
                o = put_f(o, vi[1]);
                if (d3) {
                    *o++ = ',';
                    o = put_f(o, vi[2]);
                }
            }
            if (wr) {
                *o++ = ',';
                o = put_f(o, rho[i]);
            }
            if (wp) {
                *o++ = ',';
                o = put_f(o, pres[i]);
            }
            *o++ = '\n';
            used += (size_t)(o - b);
        }
        out.resize(used);
    };
    // contiguous ranges formatted in parallel, written in order (the same bytes)
    const uint64_t n = p->ntotal;
    const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
    const uint64_t parts = std::max<uint64_t>(1, std::min<uint64_t>({(uint64_t)std::min(hw, 8u), n / 16384}));
    std::vector<std::string> chunk(parts);
    std::vector<std::thread> pool;
    for (uint64_t c = 1; c < parts; c++)
        pool.emplace_back([&, c] { lines(n * c / parts, n * (c + 1) / parts, chunk[c]); });
    lines(0, n / parts, chunk[0]);
    for (auto& t : pool) t.join();
    FILE* f = std::fopen(csv_path, "wb");
    if (!f) return set_error(RRSPH_ERR_IO, std::string("cannot write layer ") + csv_path);
    bool ok = std::fwrite(head.data(), 1, head.size(), f) == head.size();
    for (const auto& c : chunk) ok = ok && std::fwrite(c.data(), 1, c.size(), f) == c.size();
    ok = (std::fclose(f) == 0) && ok;
    if (!ok) return set_error(RRSPH_ERR_IO, std::string("short write of layer ") + csv_path);
    return RRSPH_OK;
}
