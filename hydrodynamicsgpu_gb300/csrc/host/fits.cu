// fits.cu -- minimal FITS (Flexible Image Transport System, NASA/IAU standard 4.0)
// writer: a primary header of 80-character cards and big-endian float32 data.
#include <cstdio>
#include <cstring>
#include <stdexcept>
#include <vector>

#include "fits.h"

namespace hgpu {

namespace {
void card(std::vector<char>& h, const char* key, const std::string& value) {
    char buf[81];
    std::snprintf(buf, sizeof buf, "%-8.8s= %20s", key, value.c_str());
    std::string s(buf);
    s.resize(80, ' ');
    h.insert(h.end(), s.begin(), s.end());
}
}  // namespace

bool fileExists(const std::string& path) {
    FILE* f = std::fopen(path.c_str(), "rb");
    if (!f) return false;
    std::fclose(f);
    return true;
}

void writeFitsFloat(const std::string& path, const float* data, int nx, int ny, int nz) {
    std::vector<char> h;
    card(h, "SIMPLE", "T");
    card(h, "BITPIX", "-32");
    card(h, "NAXIS", "3");
    card(h, "NAXIS1", std::to_string(nx));
    card(h, "NAXIS2", std::to_string(ny));
    card(h, "NAXIS3", std::to_string(nz));
    std::string end = "END";
    end.resize(80, ' ');
    h.insert(h.end(), end.begin(), end.end());
    h.resize((h.size() + 2879) / 2880 * 2880, ' ');
    const size_t n = (size_t)nx * ny * nz;
    std::vector<unsigned char> d(n * 4);
    for (size_t i = 0; i < n; ++i) {
        unsigned int u;
        std::memcpy(&u, data + i, 4);
        d[4 * i] = (unsigned char)(u >> 24);
        d[4 * i + 1] = (unsigned char)(u >> 16);
        d[4 * i + 2] = (unsigned char)(u >> 8);
        d[4 * i + 3] = (unsigned char)u;
    }
    d.resize((d.size() + 2879) / 2880 * 2880, 0);
    FILE* f = std::fopen(path.c_str(), "wb");
    if (!f) throw std::runtime_error("cannot open " + path + " for writing");
    bool ok = std::fwrite(h.data(), 1, h.size(), f) == h.size() && std::fwrite(d.data(), 1, d.size(), f) == d.size();
    ok = (std::fclose(f) == 0) && ok;
    if (!ok) throw std::runtime_error("write failed: " + path);
}

}  // namespace hgpu
