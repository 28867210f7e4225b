// meshio.cu -- Nek5000 mesh files on one host process (no MPI-IO).
//
// Restates the file formats of src/io.c:
//   .re2 (read_geometry, re2_header :40-63, re2_coord :65-121,
//         re2_boundary :123-210): 80-byte header "#v00x nelgt ndim nelgv",
//         float 6.54321, per element a group id and x[nv], y[nv] (, z[nv])
//         as doubles; then the curve count and 8 doubles per curve; then the
//         boundary-condition count and 8 x 8-byte records per face, of which
//         periodic faces ("P  ") are returned as (eid, fid, e1, e2).
//   .co2 (read_connectivity :212-298, parrsb_dump_con :358-425): 132-byte
//         header "#v001 nelgt nelgv nv", float test, per element
//         (element id, nv vertex ids) as int32.
//   .ma2 (parrsb_dump_map :427-505): 132-byte header "#v001 nelgt nactive
//         depth d2 npts nrnk noutflow", float test, per element
//         (part, nv vertex ids) as int32.
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <string>
#include <vector>

#include "../../include/parrsb.h"

namespace {

constexpr int RE2_HEADER = 80;
constexpr int CO2_HEADER = 132;

bool read_exact(FILE *f, void *p, size_t n) { return fread(p, 1, n, f) == n; }

std::string with_ext(const char *name, const char *ext) {
  std::string s(name);
  s += ext;
  return s;
}

int read_geometry(const char *fname, unsigned *nel, unsigned *nv, double **coord,
                  unsigned *nbcs, long long **bcs) {
  FILE *f = fopen(fname, "rb");
  if (!f) return PARRSB_ERR_ARGS;
  char hdr[RE2_HEADER + 1] = {0};
  float test = 0.f;
  if (!read_exact(f, hdr, RE2_HEADER) || !read_exact(f, &test, 4)) {
    fclose(f);
    return PARRSB_ERR_ARGS;
  }
  char version[6] = {0};
  long long nelgt = 0, nelgv = 0;
  int ndim = 0;
  if (sscanf(hdr, "%5s %lld %d %lld", version, &nelgt, &ndim, &nelgv) != 4 ||
      fabs(test - 6.543210) > 1e-7 || (ndim != 2 && ndim != 3) || nelgt < 0) {
    fclose(f);
    return PARRSB_ERR_ARGS;
  }
  unsigned n_v = ndim == 2 ? 4 : 8;
  size_t ne = (size_t)nelgt;
  double *c = (double *)calloc(ne * n_v * ndim + 1, sizeof(double));
  std::vector<double> rec(1 + n_v * ndim);
  for (size_t i = 0; i < ne; i++) {
    if (!read_exact(f, rec.data(), rec.size() * sizeof(double))) {
      free(c);
      fclose(f);
      return PARRSB_ERR_ARGS;
    }
    for (unsigned k = 0; k < n_v; k++)
      for (int d = 0; d < ndim; d++) c[i * n_v * ndim + k * ndim + d] = rec[1 + d * n_v + k];
  }
  // curves, then boundary conditions
  double t = 0.0;
  std::vector<long long> per;
  if (read_exact(f, &t, sizeof(double))) {
    long ncurves = (long)t;
    if (ncurves < 0 || fseek(f, (long)(8 * sizeof(double)) * ncurves, SEEK_CUR) != 0) {
      free(c);
      fclose(f);
      return PARRSB_ERR_ARGS;
    }
    if (read_exact(f, &t, sizeof(double))) {
      long nb = (long)t;
      for (long b = 0; b < nb; b++) {
        double r[7];
        char cbc[9] = {0};
        if (!read_exact(f, r, 7 * sizeof(double)) || !read_exact(f, cbc, 8)) break;
        if (strncmp(cbc, "P  ", 3) == 0) {
          per.push_back((long long)r[0]);
          per.push_back((long long)r[1]);
          per.push_back((long long)r[2]);
          per.push_back((long long)r[3]);
        }
      }
    }
  }
  fclose(f);
  *nel = (unsigned)ne;
  *nv = n_v;
  *coord = c;
  if (nbcs) *nbcs = (unsigned)(per.size() / 4);
  if (bcs) {
    *bcs = (long long *)calloc(per.size() + 1, sizeof(long long));
    if (!per.empty()) memcpy(*bcs, per.data(), per.size() * sizeof(long long));
  }
  return PARRSB_OK;
}

int read_connectivity(const char *fname, unsigned *nel, unsigned *nv, long long **vl) {
  FILE *f = fopen(fname, "rb");
  if (!f) return PARRSB_ERR_ARGS;
  char hdr[CO2_HEADER + 1] = {0};
  float test = 0.f;
  if (!read_exact(f, hdr, CO2_HEADER) || !read_exact(f, &test, 4)) {
    fclose(f);
    return PARRSB_ERR_ARGS;
  }
  char version[6] = {0};
  long long nelgt = 0, nelgv = 0;
  unsigned n_v = 0;
  if (sscanf(hdr, "%5s %12lld %12lld %u", version, &nelgt, &nelgv, &n_v) != 4 ||
      fabs(test - 6.543210) > 1e-7 || nelgt < 0 || n_v == 0 || n_v > 8) {
    fclose(f);
    return PARRSB_ERR_ARGS;
  }
  if ((*nv != 0 && *nv != n_v) || (*nel != 0 && *nel != (unsigned)nelgt)) {
    fclose(f);
    return PARRSB_ERR_ARGS;  // does not match the .re2 read first
  }
  long long *v = (long long *)calloc((size_t)nelgt * n_v + 1, sizeof(long long));
  std::vector<int> rec(n_v + 1);
  for (long long i = 0; i < nelgt; i++) {
    if (!read_exact(f, rec.data(), rec.size() * sizeof(int))) {
      free(v);
      fclose(f);
      return PARRSB_ERR_ARGS;
    }
    for (unsigned k = 0; k < n_v; k++) v[i * n_v + k] = rec[1 + k];
  }
  fclose(f);
  *nel = (unsigned)nelgt;
  *nv = n_v;
  *vl = v;
  return PARRSB_OK;
}

}  // namespace

extern "C" int parrsb_read_mesh(unsigned *nel, unsigned *nv, long long **vl, double **coord,
                                unsigned *nbcs, long long **bcs, char *name, int read) {
  if (!nel || !nv || !name) return PARRSB_ERR_ARGS;
  *nv = 0, *nel = 0;
  if (read & 1) {
    if (!coord) return PARRSB_ERR_ARGS;
    int rc = read_geometry(with_ext(name, ".re2").c_str(), nel, nv, coord, nbcs, bcs);
    if (rc) return rc;
  }
  if (read & 2) {
    if (!vl) return PARRSB_ERR_ARGS;
    int rc = read_connectivity(with_ext(name, ".co2").c_str(), nel, nv, vl);
    if (rc) return rc;
  }
  return PARRSB_OK;
}

extern "C" int parrsb_dump_con(char *name, unsigned nelt, unsigned nv, long long *vl) {
  if (!name || (nelt && !vl) || nv == 0 || nv > 8) return PARRSB_ERR_ARGS;
  FILE *f = fopen(with_ext(name, ".co2").c_str(), "wb");
  if (!f) return PARRSB_ERR_ARGS;
  char hdr[CO2_HEADER + 1];
  snprintf(hdr, sizeof(hdr), "%5s%12d%12d%12d", "#v001", (int)nelt, (int)nelt, (int)nv);
  memset(hdr + strlen(hdr), ' ', CO2_HEADER - strlen(hdr));
  const float test = 6.54321f;
  bool ok = fwrite(hdr, 1, CO2_HEADER, f) == CO2_HEADER && fwrite(&test, 4, 1, f) == 1;
  std::vector<int> rec(nv + 1);
  for (unsigned i = 0; i < nelt && ok; i++) {
    rec[0] = (int)(i + 1);
    for (unsigned j = 0; j < nv; j++) rec[1 + j] = (int)vl[(size_t)i * nv + j];
    ok = fwrite(rec.data(), sizeof(int), rec.size(), f) == rec.size();
  }
  ok = (fclose(f) == 0) && ok;
  return ok ? PARRSB_OK : PARRSB_ERR_ARGS;
}

extern "C" int parrsb_dump_map(char *name, unsigned nelt, unsigned nv, long long *vtx,
                               const int *part) {
  if (!name || (nelt && (!vtx || !part)) || nv == 0 || nv > 8) return PARRSB_ERR_ARGS;
  FILE *f = fopen(with_ext(name, ".ma2").c_str(), "wb");
  if (!f) return PARRSB_ERR_ARGS;
  int nelgt = (int)nelt;
  int depth = 0;
  while ((1ll << (depth + 1)) <= (long long)nelgt) depth++;  // floor(log2)
  int d2 = 1 << depth;
  char hdr[CO2_HEADER + 1];
  snprintf(hdr, sizeof(hdr), "%5s%12d%12d%12d%12d%12d%12d%12d", "#v001", nelgt, nelgt, depth,
           d2, (int)(nelgt * (int)nv), nelgt, 0);
  memset(hdr + strlen(hdr), ' ', CO2_HEADER - strlen(hdr));
  const float test = 6.54321f;
  bool ok = fwrite(hdr, 1, CO2_HEADER, f) == CO2_HEADER && fwrite(&test, 4, 1, f) == 1;
  std::vector<int> rec(nv + 1);
  for (unsigned i = 0; i < nelt && ok; i++) {
    rec[0] = part[i];
    for (unsigned j = 0; j < nv; j++) rec[1 + j] = (int)vtx[(size_t)i * nv + j];
    ok = fwrite(rec.data(), sizeof(int), rec.size(), f) == rec.size();
  }
  ok = (fclose(f) == 0) && ok;
  return ok ? PARRSB_OK : PARRSB_ERR_ARGS;
}
