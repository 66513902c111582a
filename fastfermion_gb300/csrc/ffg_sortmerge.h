// Internal interface of the sort-and-reduce rotation pass (ffg_sortmerge.cu).
#pragma once
#include <cstddef>
#include <cuda_runtime.h>

namespace ffg_sm {

typedef unsigned long long u64;

struct SmGate {
    u64 p[4];     // axis planes in store order (NW x words, then NW z words)
    double c, s;  // cos theta, sin theta
    int yP;       // popc(x_P & z_P)
    int maxdeg;   // partner filter
};

// One rotation on a dense store of n terms (kw key planes with the given
// stride).  Writes the merged terms to okey/ore/oim (capacity ocap, plane
// stride ocap) and their count to *n_out; when *n_out > ocap nothing is
// written and the caller retries with a larger output.  *emits = partners that
// passed the degree filter.  Returns 0 or a cudaError_t.  Synchronises the
// stream once (to learn *n_out).
int rotation(cudaStream_t st, int kw, bool cplx, const u64* key, const double* re, const double* im, u64 n, u64 stride,
             const SmGate& g, u64* okey, double* ore, double* oim, u64 ocap, u64* n_out, u64* emits, void** scratch,
             size_t* scratch_bytes);

}  // namespace ffg_sm
