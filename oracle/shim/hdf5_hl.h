/* Stand-in for HDF5's high-level API; no-ops (see hdf5.h). TEST INFRASTRUCTURE ONLY. */
#ifndef PSPH_SHIM_HDF5_HL_H
#define PSPH_SHIM_HDF5_HL_H
#include "hdf5.h"
static inline herr_t H5LTmake_dataset_int(hid_t, const char*, int, const hsize_t*, const int*) { return 0; }
static inline herr_t H5LTmake_dataset_float(hid_t, const char*, int, const hsize_t*, const float*) { return 0; }
static inline herr_t H5LTmake_dataset_double(hid_t, const char*, int, const hsize_t*, const double*) { return 0; }
#endif
