// output.h -- host-side writer of the reference's snapshot files (output.cpp's MPI_IO_Write,
// WriteXDMF and ASC_WRITE for one rank) from a packed [10][nz][ny][nx] FP64 snapshot.
#pragma once

#include <string>
#include <vector>

namespace mhdgb {

struct SnapshotMeta {
  std::string root;              // directory that receives bindata/ and ascdata/
  int index = 0;                 // output index (the reference's Output() counter)
  double time = 0.0, dt = 0.0;   // resolution_mod::time_sim and dt written in the headers
  bool ascii = false;            // also write ascdata/snap000-%05d.csv (config::asciiout)
  int nx = 0, ny = 0, nz = 0;
  std::vector<double> x1a, x2a, x3a;  // cell faces, itot/jtot/ktot entries from index 0
};

// Writes every file of one snapshot; returns 0, or -1 with a message in *err on an I/O failure.
int write_snapshot_files(const SnapshotMeta& m, const double* field, std::string* err);

}  // namespace mhdgb
