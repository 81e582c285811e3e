/*
 * State-directory I/O shared by the oracle drivers (TEST INFRASTRUCTURE ONLY).
 *
 * A state directory holds one raw little-endian file per per-particle field
 * (<name>.bin; int32 or float64, vector fields interleaved [i*3+d], tensors
 * row-major [i*9+r*3+c]) plus config.txt with one "key value..." line per
 * domain/integrator scalar. The Python side (persiansph_gb300/statefile.py)
 * reads and writes the same layout.
 */
#ifndef PSPH_ORACLE_STATE_IO_H
#define PSPH_ORACLE_STATE_IO_H

#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Per-particle int32 fields, in file order. */
#define PSPH_INT_FIELDS(X) \
  X(id) X(material) X(is_free) X(no_slip) X(pres_eq) X(shepard) X(les) X(vis_m) X(fail) \
  X(seepage_type) X(var_porosity) X(is_sat) X(in_out)

/* Per-particle float64 scalar fields. */
#define PSPH_F64_FIELDS(X)                                                                      \
  X(density) X(densitya) X(densityb) X(ddensity) X(pressure) X(mass) X(h) X(cs) X(p0)            \
  X(ref_density) X(fpmassc) X(alpha) X(beta) X(mu) X(mu_ref) X(t0) X(bingham_m) X(csmag) X(ti)   \
  X(tin) X(ti_init_dist) X(g_mod) X(k_mod) X(sigmay) X(cohesion) X(phi) X(psi) X(zwab) X(sumden) \
  X(sumkernel) X(shear_rate) X(sbar) X(n0) X(k) X(k2) X(d) X(rho_f) X(volume) X(s)

/* Per-particle 3-vectors. */
#define PSPH_VEC_FIELDS(X) X(x) X(v) X(va) X(vb) X(a) X(nsv) X(vxsph)

/* Per-particle 3x3 tensors. */
#define PSPH_TEN_FIELDS(X)                                                                     \
  X(sigma) X(sigmaa) X(sigmab) X(shear_stress) X(shear_stressa) X(shear_stressb) X(strain)       \
  X(straina) X(strainb) X(strain_rate) X(rotation_rate) X(tir)

static inline int psph_io_read(const char* dir, const char* name, void* buf, size_t bytes) {
  char path[4096];
  snprintf(path, sizeof path, "%s/%s.bin", dir, name);
  FILE* f = fopen(path, "rb");
  if (!f) return -1;
  size_t got = fread(buf, 1, bytes, f);
  fclose(f);
  return got == bytes ? 0 : -2;
}

static inline int psph_io_write(const char* dir, const char* name, const void* buf, size_t bytes) {
  char path[4096];
  snprintf(path, sizeof path, "%s/%s.bin", dir, name);
  FILE* f = fopen(path, "wb");
  if (!f) return -1;
  size_t put = fwrite(buf, 1, bytes, f);
  fclose(f);
  return put == bytes ? 0 : -2;
}

/* Looks up "key v0 v1 ..." in config.txt; returns the number of values read. */
static inline int psph_io_cfg(const char* dir, const char* key, double* vals, int maxv) {
  char path[4096], line[8192];
  snprintf(path, sizeof path, "%s/config.txt", dir);
  FILE* f = fopen(path, "r");
  if (!f) return 0;
  int nv = 0;
  size_t kl = strlen(key);
  while (fgets(line, sizeof line, f)) {
    if (strncmp(line, key, kl) == 0 && (line[kl] == ' ' || line[kl] == '\t')) {
      char* p = line + kl;
      while (nv < maxv) {
        char* end;
        double d = strtod(p, &end);
        if (end == p) break;
        vals[nv++] = d;
        p = end;
      }
      break;
    }
  }
  fclose(f);
  return nv;
}

static inline double psph_io_cfg1(const char* dir, const char* key, double dflt) {
  double v;
  return psph_io_cfg(dir, key, &v, 1) == 1 ? v : dflt;
}

#ifdef __cplusplus
}
#endif

#endif
