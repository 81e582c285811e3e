/*
 * Stand-in for the HDF5 C API (written for this project). The reference only
 * writes snapshots through it (Source/Domain.cpp WriteXDMF); the oracle build
 * never writes output, so every call is a no-op. TEST INFRASTRUCTURE ONLY.
 */
#ifndef PSPH_SHIM_HDF5_H
#define PSPH_SHIM_HDF5_H
typedef long long hid_t;
typedef unsigned long long hsize_t;
typedef int herr_t;
#define H5F_ACC_TRUNC 2u
#define H5P_DEFAULT 0
#define H5F_SCOPE_GLOBAL 1
static inline hid_t H5Fcreate(const char*, unsigned, hid_t, hid_t) { return 1; }
static inline herr_t H5Fflush(hid_t, int) { return 0; }
static inline herr_t H5Fclose(hid_t) { return 0; }
#endif
