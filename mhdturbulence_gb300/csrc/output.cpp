// output.cpp -- the reference's snapshot files written from a packed FP64 snapshot.
//
// For one rank the reference's Output() (src_cpp_kokkos_host/output.cpp:379-407) writes, under the
// working directory:
//   bindata/unf%05d.dat    "# time dt" (%.17g) and the three interior extents   (MPI_IO_Write, 88-98)
//   bindata/grid{1,2,3}D.bin  [2][n+1] FP64: cell centres x?b then faces x?a from index ngh (215-236)
//   bindata/field%05d.bin  [10][nz][ny][nx] FP64: d v1 v2 v3 b1 b2 b3 bp p X1 (247-260, 184-200)
//   bindata/field%05d.xmf  XDMF 2.0 description of the two binaries              (WriteXDMF, 273-343)
//   ascdata/snap000-%05d.csv  plane k = ngh: x y d vx vy p X1 at %.6e            (ASC_WRITE, 348-386)
// Here the same bytes come from the snapshot the device packed (k_snapshot), so the host only
// formats and writes.  The grid files are rewritten with every snapshot (the reference writes them
// with its first one; the content is the same).
#include "output.h"

#include <sys/stat.h>

#include <cerrno>
#include <cstdarg>
#include <cstdio>
#include <cstring>

namespace mhdgb {
namespace {

constexpr int kNgh = 2;
const char* const kNames[10] = {"d", "v1", "v2", "v3", "b1", "b2", "b3", "bp", "p", "X1"};

bool make_dirs(const std::string& path, std::string* err) {
  std::string cur;
  size_t pos = 0;
  while (pos != std::string::npos) {
    pos = path.find('/', pos + 1);
    cur = path.substr(0, pos);
    if (cur.empty()) continue;
    if (mkdir(cur.c_str(), 0777) != 0 && errno != EEXIST) {
      *err = "cannot create " + cur + ": " + std::strerror(errno);
      return false;
    }
  }
  return true;
}

struct File {
  FILE* fp = nullptr;
  std::string name;
  bool ok = true;
  File(const std::string& n, const char* mode) : name(n) { fp = std::fopen(n.c_str(), mode); ok = fp != nullptr; }
  ~File() { close(); }
  bool close() {
    if (fp && std::fclose(fp) != 0) ok = false;
    fp = nullptr;
    return ok;
  }
  void write(const void* p, size_t bytes) {
    if (ok && std::fwrite(p, 1, bytes, fp) != bytes) ok = false;
  }
  void printf(const char* fmt, ...) __attribute__((format(printf, 2, 3)));
};

void File::printf(const char* fmt, ...) {
  if (!ok) return;
  va_list ap;
  va_start(ap, fmt);
  if (std::vfprintf(fp, fmt, ap) < 0) ok = false;
  va_end(ap);
}

bool done(File& f, std::string* err) {
  if (f.close()) return true;
  *err = "cannot write " + f.name + ": " + std::strerror(errno);
  return false;
}

double centre(const std::vector<double>& xa, int i) { return 0.5e0 * (xa[i + 1] + xa[i]); }

}  // namespace

int write_snapshot_files(const SnapshotMeta& m, const double* field, std::string* err) {
  const std::string root = m.root.empty() ? std::string(".") : m.root;
  const std::string bdir = root + "/bindata/", adir = root + "/ascdata/";
  if (!make_dirs(root + "/bindata", err)) return -1;
  char name[64];
  const long long ncell = (long long)m.nx * m.ny * m.nz;

  std::snprintf(name, sizeof(name), "unf%05d.dat", m.index);
  {
    File f(bdir + name, "w");
    f.printf("# %.17g %.17g\n", m.time, m.dt);
    f.printf("# %d \n# %d \n# %d \n", m.nx, m.ny, m.nz);
    if (!done(f, err)) return -1;
  }
  const std::vector<double>* axes[3] = {&m.x1a, &m.x2a, &m.x3a};
  const int ns[3] = {m.nx, m.ny, m.nz};
  for (int d = 0; d < 3; d++) {
    const int n1 = ns[d] + 1;
    std::vector<double> g(2 * (size_t)n1);
    for (int i = 0; i < n1; i++) {
      g[i] = centre(*axes[d], kNgh + i);
      g[n1 + i] = (*axes[d])[kNgh + i];
    }
    std::snprintf(name, sizeof(name), "grid%dD.bin", d + 1);
    File f(bdir + name, "wb");
    f.write(g.data(), g.size() * sizeof(double));
    if (!done(f, err)) return -1;
  }
  std::snprintf(name, sizeof(name), "field%05d.bin", m.index);
  const std::string fdata = name;
  {
    File f(bdir + fdata, "wb");
    f.write(field, (size_t)ncell * 10 * sizeof(double));
    if (!done(f, err)) return -1;
  }
  std::snprintf(name, sizeof(name), "field%05d.xmf", m.index);
  {
    File f(bdir + name, "w");
    f.printf("<?xml version=\"1.0\" ?>\n<!DOCTYPE Xdmf SYSTEM \"Xdmf.dtd\" []>\n<Xdmf Version=\"2.0\">\n");
    f.printf("  <Domain>\n    <Grid Name=\"Grid\" GridType=\"Uniform\">\n");
    f.printf("      <Time Value=\"%.16e\"/>\n", m.time);
    f.printf("      <Topology TopologyType=\"3DRectMesh\" Dimensions=\"%d %d %d\"/>\n", m.nz + 1, m.ny + 1, m.nx + 1);
    f.printf("      <Geometry GeometryType=\"VXVYVZ\">\n");
    for (int d = 0; d < 3; d++)
      f.printf("        <DataItem Dimensions=\"%d\" NumberType=\"Float\" Precision=\"8\" Format=\"Binary\" "
               "Endian=\"Little\" Seek=\"%lld\">grid%dD.bin</DataItem>\n",
               ns[d] + 1, (long long)(ns[d] + 1) * 8, d + 1);
    f.printf("      </Geometry>\n");
    for (int v = 0; v < 10; v++) {
      f.printf("      <Attribute Name=\"%s\" AttributeType=\"Scalar\" Center=\"Cell\">\n", kNames[v]);
      f.printf("        <DataItem Dimensions=\"%d %d %d\" NumberType=\"Float\" Precision=\"8\" Format=\"Binary\" "
               "Endian=\"Little\" Seek=\"%lld\">%s</DataItem>\n",
               m.nz, m.ny, m.nx, (long long)v * ncell * 8, fdata.c_str());
      f.printf("      </Attribute>\n");
    }
    f.printf("    </Grid>\n  </Domain>\n</Xdmf>\n");
    if (!done(f, err)) return -1;
  }
  if (m.ascii) {
    if (!make_dirs(root + "/ascdata", err)) return -1;
    std::snprintf(name, sizeof(name), "snap%03d-%05d.csv", 0, m.index);
    File f(adir + name, "w");
    f.printf("# %.6e %.6e\n# %d\n# %d\n", m.time, m.dt, m.nx, m.ny);
    f.printf("# %d %.6e\n", kNgh, centre(m.x3a, kNgh));
    f.printf("# x y d vx vy p X1\n");
    // plane k = ngh is the first plane of the snapshot; its variables 0, 1, 2, 8, 9 are d vx vy p X1
    for (int j = 0; j < m.ny; j++) {
      for (int i = 0; i < m.nx; i++) {
        const size_t c = (size_t)j * m.nx + i;
        f.printf("%.6e %.6e %.6e %.6e %.6e %.6e %.6e\n", centre(m.x1a, kNgh + i), centre(m.x2a, kNgh + j),
                 field[0 * ncell + c], field[1 * ncell + c], field[2 * ncell + c], field[8 * ncell + c],
                 field[9 * ncell + c]);
      }
      f.printf("\n");
    }
    if (!done(f, err)) return -1;
  }
  return 0;
}

}  // namespace mhdgb
