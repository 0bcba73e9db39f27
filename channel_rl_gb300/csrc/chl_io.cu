// Snapshot and parameter-file I/O in the reference's formats (host code).
//
// Snapshot (output_data, input_output.f90:593-730; read_input_data,
// :390-560; the layout scripts/check_file.m reads): a stream of
//   int32 nx,  float64 x(1:nx)      int32 ny,  float64 y(1:ny)
//   int32 nz,  float64 z(1:nz)      int32 nx-1, float64 xm(1:nx-1)
//   int32 ny-1, float64 ym(1:ny-1)  int32 nz-1, float64 zm(1:nz-1)
//   int32[3] (nx, nyg, nzg),  float64 U   (Fortran order, all z planes)
//   int32[3] (nxg, ny, nzg),  float64 V
//   int32[3] (nxg, nyg, nz),  float64 W
//   [int32[3] (nxg, nyg, nzg), float64 P]      written by output_data
//   [int32[3] (nxg, nyg, nzg), float64 nu_t]
// little-endian, no record markers (access='stream').  The planes the
// reference writes rank by rank add up to the whole global array in a
// multi-rank run, which is what is read and written here.  xm are the cell
// centres 0.5 (x(i) + x(i+1)) (initialization.f90:194-200).
//
// Parameter file (read_input_parameters, input_output.f90:20-91): comment
// lines alternating with values, list-directed.
//
// Errors come back as status codes with a message (chl_io_last_error), where
// the reference stops the program.
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/chl.h"

namespace {

std::mutex g_err_mu;
std::string g_err;

int fail(int code, const std::string& msg) {
  std::lock_guard<std::mutex> lk(g_err_mu);
  g_err = msg;
  return code;
}

bool little_endian() {
  const uint16_t one = 1;
  unsigned char b;
  std::memcpy(&b, &one, 1);
  return b == 1;
}

void swap_bytes(void* p, size_t size, size_t n) {
  unsigned char* c = static_cast<unsigned char*>(p);
  for (size_t i = 0; i < n; ++i, c += size)
    for (size_t a = 0, b = size - 1; a < b; ++a, --b) std::swap(c[a], c[b]);
}

// All file integers and reals are little-endian.
bool put(FILE* f, const void* p, size_t size, size_t n) {
  if (little_endian()) return std::fwrite(p, size, n, f) == n;
  std::vector<unsigned char> tmp(size * n);
  std::memcpy(tmp.data(), p, size * n);
  swap_bytes(tmp.data(), size, n);
  return std::fwrite(tmp.data(), size, n, f) == n;
}

bool get(FILE* f, void* p, size_t size, size_t n) {
  if (std::fread(p, size, n, f) != n) return false;
  if (!little_endian()) swap_bytes(p, size, n);
  return true;
}

struct File {
  FILE* f = nullptr;
  ~File() { if (f) std::fclose(f); }
};

bool put_vec(FILE* f, const double* a, int32_t n) { return put(f, &n, 4, 1) && put(f, a, 8, (size_t)n); }

bool put_field(FILE* f, const double* a, int32_t n1, int32_t n2, int32_t n3) {
  const int32_t d[3] = {n1, n2, n3};
  return put(f, d, 4, 3) && put(f, a, 8, (size_t)n1 * n2 * n3);
}

}  // namespace

extern "C" {

const char* chl_io_last_error(void) {
  std::lock_guard<std::mutex> lk(g_err_mu);
  return g_err.c_str();
}

int chl_snapshot_dims(const char* path, int* nx, int* ny, int* nz) {
  if (!path || !nx || !ny || !nz) return fail(CHL_E_ARG, "snapshot: null argument");
  File F;
  F.f = std::fopen(path, "rb");
  if (!F.f) return fail(CHL_E_IO, std::string("snapshot: cannot open ") + path);
  int32_t n[3];
  for (int a = 0; a < 3; ++a) {
    if (!get(F.f, &n[a], 4, 1) || n[a] < 2 || n[a] > (1 << 24))
      return fail(CHL_E_IO, "snapshot: bad mesh header");
    if (std::fseek(F.f, 8L * n[a], SEEK_CUR) != 0) return fail(CHL_E_IO, "snapshot: truncated mesh");
  }
  *nx = n[0]; *ny = n[1]; *nz = n[2];
  return CHL_OK;
}

int chl_snapshot_write(const char* path, int nx, int ny, int nz, const double* x, const double* y,
                       const double* z, const double* U, const double* V, const double* W,
                       const double* P, const double* nu_t) {
  if (!path || !x || !y || !z || !U || !V || !W) return fail(CHL_E_ARG, "snapshot: null argument");
  if (nx < 2 || ny < 2 || nz < 2) return fail(CHL_E_ARG, "snapshot: bad extents");
  if ((P == nullptr) != (nu_t == nullptr)) return fail(CHL_E_ARG, "snapshot: P and nu_t go together");
  const int nxg = nx + 1, nyg = ny + 1, nzg = nz + 1;
  std::vector<double> xm(nx - 1), ym(ny - 1), zm(nz - 1);
  for (int i = 0; i < nx - 1; ++i) xm[i] = 0.5 * (x[i] + x[i + 1]);
  for (int j = 0; j < ny - 1; ++j) ym[j] = 0.5 * (y[j] + y[j + 1]);
  for (int k = 0; k < nz - 1; ++k) zm[k] = 0.5 * (z[k] + z[k + 1]);
  File F;
  F.f = std::fopen(path, "wb");
  if (!F.f) return fail(CHL_E_IO, std::string("snapshot: cannot create ") + path);
  bool ok = put_vec(F.f, x, nx) && put_vec(F.f, y, ny) && put_vec(F.f, z, nz) &&
            put_vec(F.f, xm.data(), nx - 1) && put_vec(F.f, ym.data(), ny - 1) && put_vec(F.f, zm.data(), nz - 1) &&
            put_field(F.f, U, nx, nyg, nzg) && put_field(F.f, V, nxg, ny, nzg) && put_field(F.f, W, nxg, nyg, nz);
  if (ok && P) ok = put_field(F.f, P, nxg, nyg, nzg) && put_field(F.f, nu_t, nxg, nyg, nzg);
  if (!ok) return fail(CHL_E_IO, std::string("snapshot: write failed for ") + path);
  if (std::fclose(F.f) != 0) { F.f = nullptr; return fail(CHL_E_IO, "snapshot: close failed"); }
  F.f = nullptr;
  return CHL_OK;
}

int chl_snapshot_read(const char* path, int nx, int ny, int nz, double* x, double* y, double* z,
                      double* U, double* V, double* W) {
  if (!path || !x || !y || !z || !U || !V || !W) return fail(CHL_E_ARG, "snapshot: null argument");
  File F;
  F.f = std::fopen(path, "rb");
  if (!F.f) return fail(CHL_E_IO, std::string("snapshot: cannot open ") + path);
  const int nxg = nx + 1, nyg = ny + 1, nzg = nz + 1;
  auto vec = [&](double* dst, int n, const char* what) -> int {
    int32_t m;
    if (!get(F.f, &m, 4, 1)) return fail(CHL_E_IO, std::string("snapshot: truncated at ") + what);
    if (m != n) return fail(CHL_E_ARG, std::string("snapshot: ") + what + " size " + std::to_string(m) +
                                       " /= " + std::to_string(n));
    if (dst) { if (!get(F.f, dst, 8, (size_t)n)) return fail(CHL_E_IO, std::string("snapshot: truncated ") + what); }
    else if (std::fseek(F.f, 8L * n, SEEK_CUR) != 0) return fail(CHL_E_IO, "snapshot: truncated");
    return CHL_OK;
  };
  auto field = [&](double* dst, int n1, int n2, int n3, const char* what) -> int {
    int32_t d[3];
    if (!get(F.f, d, 4, 3)) return fail(CHL_E_IO, std::string("snapshot: truncated at ") + what);
    if (d[0] != n1 || d[1] != n2 || d[2] != n3)
      return fail(CHL_E_ARG, std::string("snapshot: wrong size in input file (") + what + ")");
    if (!get(F.f, dst, 8, (size_t)n1 * n2 * n3)) return fail(CHL_E_IO, std::string("snapshot: truncated ") + what);
    return CHL_OK;
  };
  int rc;
  if ((rc = vec(x, nx, "nx")) || (rc = vec(y, ny, "ny")) || (rc = vec(z, nz, "nz")) ||
      (rc = vec(nullptr, nx - 1, "nxm")) || (rc = vec(nullptr, ny - 1, "nym")) || (rc = vec(nullptr, nz - 1, "nzm")))
    return rc;
  if ((rc = field(U, nx, nyg, nzg, "U")) || (rc = field(V, nxg, ny, nzg, "V")) || (rc = field(W, nxg, nyg, nz, "W")))
    return rc;
  return CHL_OK;
}

int chl_read_parameters(const char* path, chl_parameters* out) {
  if (!path || !out) return fail(CHL_E_ARG, "parameters: null argument");
  File F;
  F.f = std::fopen(path, "r");
  if (!F.f) return fail(CHL_E_IO, std::string("parameters: cannot open ") + path);
  std::vector<std::string> vals;
  char line[1024];
  bool comment = true;                 // the file alternates comment and value lines
  while (std::fgets(line, sizeof line, F.f)) {
    std::string s(line);
    while (!s.empty() && (s.back() == '\n' || s.back() == '\r')) s.pop_back();
    if (s.find_first_not_of(" \t") == std::string::npos) continue;
    if (!comment) vals.push_back(s);
    comment = !comment;
  }
  if (vals.size() < 11) return fail(CHL_E_ARG, "parameters: expected 11 value lines, found " + std::to_string(vals.size()));
  chl_parameters p;
  std::memset(&p, 0, sizeof p);
  auto unq = [](const std::string& s, char* dst, size_t cap) {
    size_t a = s.find_first_not_of(" \t"), b = s.find_last_not_of(" \t");
    std::string t = s.substr(a, b - a + 1);
    if (t.size() >= 2 && (t[0] == '\'' || t[0] == '"') && t.back() == t[0]) t = t.substr(1, t.size() - 2);
    std::snprintf(dst, cap, "%s", t.c_str());
  };
  // Fortran reals may carry a 'd' exponent
  auto fix = [](std::string s) { for (char& c : s) if (c == 'd' || c == 'D') c = 'e'; return s; };
  bool ok = std::sscanf(vals[0].c_str(), "%d %d %d", &p.nx, &p.ny, &p.nz) == 3 &&
            std::sscanf(fix(vals[1]).c_str(), "%lf", &p.CFL) == 1 &&
            std::sscanf(fix(vals[2]).c_str(), "%lf", &p.nu) == 1 &&
            std::sscanf(fix(vals[3]).c_str(), "%lf %d", &p.dPdx, &p.x_mass_cte) == 2 &&
            std::sscanf(vals[4].c_str(), "%d", &p.LES_model) == 1 &&
            std::sscanf(vals[5].c_str(), "%d %d %d %d", &p.nsteps, &p.nsave, &p.nstats, &p.nmonitor) == 4 &&
            std::sscanf(vals[8].c_str(), "%d", &p.nstep_init) == 1 &&
            std::sscanf(vals[9].c_str(), "%d", &p.random_init) == 1 &&
            std::sscanf(vals[10].c_str(), "%d", &p.Dirichlet_nu_t) == 1;
  if (!ok) return fail(CHL_E_ARG, "parameters: unreadable value line");
  unq(vals[6], p.filein, sizeof p.filein);
  unq(vals[7], p.fileout, sizeof p.fileout);
  *out = p;
  return CHL_OK;
}

}  // extern "C"
