// State of a batched multi-view setup (batch.cu).
#pragma once

#include "pt_common.cuh"

namespace vcr {

struct BatchState {
  std::vector<vcr_view_desc> views;
  std::vector<BatchView> table;   // host copy of d_views
  std::vector<uint64_t> pix0;     // first pixel of each view
  BatchView* d_views = nullptr;
  double* d_sum = nullptr;        // FP64 RGB sums of all views, view after view
  uint32_t* d_ctr = nullptr;      // [0] pass counter of graph replays, [1] always 0
  uint64_t pixels = 0;
  uint32_t passes = 0;
  uint64_t samples = 0;           // camera samples per pixel summed over passes
  cudaStream_t capture = nullptr; // stream the graph is captured on
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  uint32_t graph_spp = 0;
  uint32_t table_spp = 0;         // spp the device table's path0 were written for
};

}  // namespace vcr
