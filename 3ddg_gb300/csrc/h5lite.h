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

// Reads the numeric dataset ``name`` of the root group, converted to double,
// row-major.  Reads what this writer and the HDF5 library's default
// (earliest-format) files hold: superblock version 0 or 1, version-1 object
// headers (with continuation blocks), a symbol-table root group, contiguous or
// compact layout, no filters, IEEE float (4/8 bytes) or integer (1-8 bytes) of
// either byte order.  Returns 0, or the codes of the reference's reader
// (cppsrc/HDF5Functions.cpp:398-463) by failure class: -1 file (cannot open,
// not HDF5, unsupported superblock or group structure), -2 dataset (no such
// name, unsupported object header, chunked or filtered layout), -3 dataspace
// (rank above 32, null dataspace, data outside the file), -4 datatype (not
// an integer or IEEE float).  ``type_class`` (may be null) receives the HDF5
// datatype class: 0 integer, 1 floating point.  ``why`` receives a message.
int h5_read(const std::string& path, const std::string& name, std::vector<uint64_t>& dims,
            std::vector<double>& data, int* type_class, std::string* why);

}  // namespace dg
