// Library-free writer for the HDF5 files of the reference's snapshots.
//
// The reference writes each snapshot dataset with the HDF5 C++ API
// (cppsrc/HDF5Functions.cpp:249-397): one file per dataset, a root group
// holding the named float64 dataset (contiguous, native little-endian
// double) and a one-element float64 dataset "time".  No HDF5 library exists on
// the target machines, so this writer emits that structure directly in the
// HDF5 file format: superblock version 0, version-1 object headers, a
// symbol-table root group (v1 B-tree + local heap + one symbol-table node) and
// contiguous data layout (layout message version 3).
#pragma once

#include <cstdint>
#include <string>
#include <vector>

namespace dg {

struct H5Dataset {
    std::string name;
    std::vector<uint64_t> dims;
    const double* data;  // prod(dims) doubles, row-major
};

// Returns 0 on success, -1 if the file cannot be created or written
// (the reference's FileIException code).
int h5_write(const std::string& path, const std::vector<H5Dataset>& sets);

}  // namespace dg
