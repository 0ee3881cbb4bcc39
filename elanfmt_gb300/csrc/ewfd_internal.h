// ewfd_internal.h -- declarations shared by the translation units of libewfd.so (not installed).
#pragma once
#include <vector>

#include "ewfd.h"

// Records a formatted message for ewf_last_error() and returns `status`.
int ewf_fail(int status, const char *fmt, ...);
// Extents of a field id in the reference layout; false for an id this model/damping lacks.
bool ewf_field_extent(const ewf_params &p, int id, int *ex, int *ey, int *ez);
const char *ewf_workdir(const ewf_handle *h);
int ewf_nrec(const ewf_handle *h);
int ewf_esz(const ewf_handle *h);
const double *ewf_stf_host_copy(const ewf_handle *h, std::vector<double> &out);
// True when div_spacing's reciprocal path (ewfd_kernels.cuh) reproduces IEEE division by the
// float spacing d on the current device (checked once per device and value, then cached).
bool ewf_fdiv_verified(float d);
// Writes `bytes` raw bytes to path (status code; message via ewf_last_error on failure).
int ewf_write_raw_file(const char *path, const void *data, size_t bytes);
