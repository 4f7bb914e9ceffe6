// Per-phase accounting of the library's kernels: launch counts (always) and,
// when enabled, CUDA-event durations plus the algorithmic FLOPs / bytes that
// each launch processes.  Events are recorded on the launching stream.
#pragma once
#include <vector>
#include "common.cuh"

namespace mnpbem {

enum Phase {
  PH_ASSEMBLE = 0,  // k_asm_far + k_asm_near
  PH_GEMM_BIG,      // O(n^3) complex GEMMs (Gauss-Jordan trailing updates, Sigma products)
  PH_GEMM_SMALL,    // panel GEMMs of the block inversion and the thin GEMMs of the chain / residual
  PH_BLOCKINV,      // shared-memory pivot-block inversions
  PH_ELEMWISE,      // Sigma stage, chain steps, conversions, excitation
  PH_SPECTRA,       // far fields + cross sections
  PH_GEOMETRY,      // one-time geometry / refinement set-up
  PH_HMAT_BUILD,    // H-matrices: full blocks and ACA of the far blocks
  PH_HMAT_MV,       // H-matrix products of the iterative solver
  PH_COUNT
};

struct PhaseAcc {
  double ms = 0, flops = 0, bytes = 0;
  int64_t launches = 0;
};

struct Profiler {
  bool enabled = false;
  PhaseAcc acc[PH_COUNT];
  struct Pending { cudaEvent_t a, b; int ph; double flops, bytes; int64_t launches; };
  std::vector<Pending> pending;
  std::vector<cudaEvent_t> pool;
  // graphs replayed since the last flush: their event pairs and launch counts
  struct GraphRec {
    std::vector<Pending> events;
    PhaseAcc counts[PH_COUNT];
  };
  std::vector<const GraphRec*> replayed;

  cudaEvent_t get_event() {
    if (!pool.empty()) { cudaEvent_t e = pool.back(); pool.pop_back(); return e; }
    cudaEvent_t e;
    cudaEventCreate(&e);
    return e;
  }
  int64_t timing_failures = 0;   // event pairs whose elapsed time could not be read
  bool elapsed(cudaEvent_t a, cudaEvent_t b, float& ms) {
    if (cudaEventSynchronize(b) == cudaSuccess && cudaEventElapsedTime(&ms, a, b) == cudaSuccess) return true;
    cudaGetLastError();   // a failed timing query must not surface as a later launch error
    ++timing_failures;
    return false;
  }
  void flush() {
    for (auto& p : pending) {
      float ms = 0;
      if (elapsed(p.a, p.b, ms)) acc[p.ph].ms += ms;
      pool.push_back(p.a);
      pool.push_back(p.b);
    }
    pending.clear();
    for (const GraphRec* g : replayed) {
      for (const auto& p : g->events) {
        float ms = 0;
        if (elapsed(p.a, p.b, ms)) acc[p.ph].ms += ms;
      }
      for (int q = 0; q < PH_COUNT; ++q) {
        acc[q].launches += g->counts[q].launches;
        acc[q].flops += g->counts[q].flops;
        acc[q].bytes += g->counts[q].bytes;
      }
    }
    replayed.clear();
  }
  // a capture profiler hands its events and counts to a graph record
  void move_to(GraphRec& g) {
    g.events.swap(pending);
    pending.clear();
    for (int q = 0; q < PH_COUNT; ++q) { g.counts[q] = acc[q]; acc[q] = PhaseAcc(); }
  }
  static void release(GraphRec& g) {
    for (auto& p : g.events) { cudaEventDestroy(p.a); cudaEventDestroy(p.b); }
    g.events.clear();
  }
  void reset() {
    flush();
    for (auto& a : acc) a = PhaseAcc();
    timing_failures = 0;
  }
  ~Profiler() {
    flush();
    for (auto e : pool) cudaEventDestroy(e);
  }
};

// the profiler of the handle that the current API call works on
Profiler*& current_profiler();

struct ProfScope {
  // inside a stream capture only an "external" record becomes a graph node that
  // timestamps the event on every replay (a plain record is just an edge)
  void record(cudaEvent_t e) {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    cudaStreamIsCapturing(st, &cs);
    if (cs == cudaStreamCaptureStatusActive) cudaEventRecordWithFlags(e, st, cudaEventRecordExternal);
    else cudaEventRecord(e, st);
  }
  Profiler* p;
  cudaStream_t st;
  int ph;
  double flops, bytes;
  int64_t launches;
  cudaEvent_t a = nullptr;
  ProfScope(int phase, cudaStream_t s, double fl = 0, double by = 0, int64_t nl = 1)
      : p(current_profiler()), st(s), ph(phase), flops(fl), bytes(by), launches(nl) {
    if (p && p->enabled) {
      a = p->get_event();
      record(a);
    }
  }
  ~ProfScope() {
    if (!p) return;
    p->acc[ph].launches += launches;
    p->acc[ph].flops += flops;
    p->acc[ph].bytes += bytes;
    if (p->enabled && a) {
      cudaEvent_t b = p->get_event();
      record(b);
      p->pending.push_back({a, b, ph, 0, 0, 0});
    }
  }
};

}  // namespace mnpbem
