// fits.h -- minimal FITS writer for Solver::save (src/Solver/Solver.cpp:563-589).
#pragma once
#include <string>

namespace hgpu {
// One primary HDU of 32-bit IEEE floats (BITPIX = -32), NAXIS = 3 (nx, ny, nz), x fastest,
// big-endian, header and data padded to 2880-byte records.  Throws on I/O failure.
void writeFitsFloat(const std::string& path, const float* data, int nx, int ny, int nz);
bool fileExists(const std::string& path);
}  // namespace hgpu
