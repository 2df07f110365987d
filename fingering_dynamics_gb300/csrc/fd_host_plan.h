// The chunk plan of the host-resident step (fd_host_step.cu), plain C++ so
// that it can be checked without a GPU.
#pragma once

#include <algorithm>
#include <vector>

namespace fd {

constexpr int kStripRows = 16;   // strip height of the chunked launches
constexpr int kMaxChunks = 256;  // chunks per call (bounds the events in use)

// Chunks of about chunk_rows rows (<= 0: about 1/16 of the lattice), whole
// strips of R rows, after a ramp of 1, 1, 2, 4 strips: chunk c is strips
// cb[c] .. cb[c+1]-1.  `order` is the order the chunks are computed in: those
// whose row neighbours do not wrap first (1 .. K-2), then K-1 and 0.  Chunk c
// of that order reads rows cb[c]*R - 2 .. cb[c+1]*R + 1 (wrapped), all
// uploaded once chunk `need[c]` has landed (uploads go in order 0 .. K-1).
struct HostPlan {
  int R = 0, nstrips = 0;
  std::vector<int> cb, order, need;
};

inline HostPlan host_plan(int H, int chunk_rows) {
  HostPlan p;
  p.R = H < kStripRows ? H : kStripRows;
  p.nstrips = (H + p.R - 1) / p.R;
  int m = chunk_rows > 0 ? (chunk_rows + p.R - 1) / p.R : (p.nstrips + 15) / 16;
  if (m < 1) m = 1;
  if ((p.nstrips + m - 1) / m > kMaxChunks - 4) m = (p.nstrips + kMaxChunks - 5) / (kMaxChunks - 4);
  p.cb.push_back(0);
  for (int sz : {1, 1, 2, 4})
    if (p.cb.back() < p.nstrips) p.cb.push_back(std::min(p.cb.back() + std::min(sz, m), p.nstrips));
  while (p.cb.back() < p.nstrips) p.cb.push_back(std::min(p.cb.back() + m, p.nstrips));
  const int K = (int)p.cb.size() - 1;
  for (int c = 1; c + 1 < K; ++c) p.order.push_back(c);
  if (K > 1) p.order.push_back(K - 1);
  p.order.push_back(0);
  p.need.resize(K);
  for (int c = 0; c < K; ++c) p.need[c] = (c >= 1 && c + 1 < K) ? c + 1 : K - 1;
  return p;
}

}  // namespace fd
