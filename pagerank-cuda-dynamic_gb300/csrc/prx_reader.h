// prx_reader.h -- the buffered file reader shared by the host edge-list
// parser (prx_io.cpp) and the device one (prx_parse.cu).
#pragma once
#include <cstdint>
#include <cstdio>
#include <vector>

struct prx_edge_reader {
  FILE* f = nullptr;
  std::vector<char> buf;
  size_t beg = 0, end = 0;  // unread bytes: buf[beg .. end)
  bool eof = false;
};

namespace prx_io {
// Move the unread bytes to the front and read more (the buffer doubles when a
// single line fills it).  Sets eof when nothing more could be read.
void fill(prx_edge_reader* r);
// MatrixMarket header (readMtxHeader, inc/mtx.hxx:39-54): *order = max(rows,
// cols), 0 for a file that is not "matrix coordinate"; *symmetric for
// symmetric and skew-symmetric files.  Leaves r at the first entry line.
int mtx_header(prx_edge_reader* r, uint64_t* order, bool* symmetric);
}  // namespace prx_io
