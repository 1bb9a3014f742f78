// Persistent 2D forward of a small batch: one cooperative launch runs every time step
// (persist2d.cu).
#pragma once
#include "common.cuh"

namespace sa {

#ifndef SA_PERSIST_THREADS
#define SA_PERSIST_THREADS 512
#endif
constexpr int PERSIST_THREADS = SA_PERSIST_THREADS;

// Arguments of the persistent forward. Step t reads p[t] from f1 (t odd) or f0 and writes p[t+1]
// in place of p[t-1], as the step passes do.
struct Persist2D {
    Step2D s;                    // grid, pitch, shot stride, medium, weights (field pointers unused)
    float* f0;
    float* f1;
    int nt;                      // steps 1 .. nt-2
    int tx, ty;                  // tile rows and columns of a CTA (ty even)
    int tiles_x, tiles_y;        // tiles of one shot pair; CTA b: pair b / (tiles_x tiles_y)
    // source injection by target point (Targets of the plan), each target applied by the CTA that
    // owns its point: CTA b applies targets cta_tgt[cta_off[b] .. cta_off[b+1])
    const int* cta_off;
    const int* cta_tgt;
    const long long* tidx;
    const int* toff;
    const float* tcoef;
    const int* tpoint;
    const float* src_amp;        // [nt][n_src]
    int n_src;
    const Gather* gat;           // receivers, each gathered by the CTA holding its base corner
    int n_rec;
    float* rec_amp;              // [nt][n_rec]
    int* flag;                   // per CTA: the last step whose tile of p[t+1] is stored (zero before the launch)
    int* err;                    // set to 1 when a flag wait gives up (zero before the launch)
    int extra;                   // steps a wait asks for beyond the one it needs (nonzero only to test the timeout)
    long long spin_limit;        // polls of a flag wait before it gives up
};

// Shared memory of a CTA with tiles of tx x ty points; co-resident CTAs per SM of that size.
size_t persist2d_smem(int kind, bool ot4, int tx, int ty);
int persist2d_blocks_per_sm(int kind, bool ot4, size_t smem);
// Cooperative launch of nblocks CTAs.
cudaError_t launch_persist2d(int kind, bool ot4, int nblocks, size_t smem, cudaStream_t s, const Persist2D& a);

}  // namespace sa
