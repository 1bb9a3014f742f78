// Persistent 2D forward of a small batch: one cooperative launch runs every time step
// (persist2d.cu).
#pragma once
#include "common.cuh"

namespace sa {

#ifndef SA_PERSIST_THREADS
#define SA_PERSIST_THREADS 384
#endif
constexpr int PERSIST_THREADS = SA_PERSIST_THREADS;
// rows of one column a thread computes in the first (l) and the second (update) stencil stage
#ifndef PERSIST_NR1
#define PERSIST_NR1 4
#endif
#ifndef PERSIST_NR2
#define PERSIST_NR2 2
#endif
// shared-memory slots of a CTA's source values at a step: a CTA with more targets adds them to
// the new level in a pass of its own
constexpr int PERSIST_SRC_SLOTS = 64;
// halo lines a thread has in flight at once
#ifndef SA_PERSIST_BATCH
#define SA_PERSIST_BATCH 4
#endif
constexpr int PERSIST_BATCH = SA_PERSIST_BATCH;
// memory semantics of the exchange lines' loads and stores
#ifndef PERSIST_LINE_SEM
#define PERSIST_LINE_SEM "relaxed.gpu"
#endif
// between polls of lines that do not hold their level yet
#ifndef PERSIST_POLL_PAUSE
#define PERSIST_POLL_PAUSE __nanosleep(20)
#endif

// Arguments of the persistent forward.
struct Persist2D {
    Step2D s;                    // grid, pitch, shot stride, medium, weights (field pointers unused)
    uint4* xch;                  // exchange lines: slot (level & 1), pair, point x pitch + y (zero before the launch)
    long long xch_slot;          // lines per slot
    int nt;                      // steps 1 .. nt-2
    int tx, ty;                  // tile rows and columns of a CTA (ty even)
    int tiles_x, tiles_y;        // tiles of one shot pair; CTA b: pair b / (tiles_x tiles_y)
    // source injection by target point (Targets of the plan), each target applied by the CTA that
    // owns its point: CTA b applies targets cta_tgt[cta_off[b] .. cta_off[b+1]). The owner first
    // sums each target's entries for every step into srcv[(cta_off[b] + j) nt + t].
    const int* cta_off;
    const int* cta_tgt;
    const long long* tidx;
    const int* toff;
    const float* tcoef;
    const int* tpoint;
    const float* src_amp;        // [nt][n_src]
    int n_src;
    float* srcv;                 // [targets][nt]
    // receivers, each gathered by the CTA holding its base corner: CTA b gathers
    // gat[rec_idx[rec_off[b] .. rec_off[b+1])]
    const int* rec_off;
    const int* rec_idx;
    const Gather* gat;
    int n_rec;
    float* rec_amp;              // [nt][n_rec]
    int* err;                    // set to 1 when a wait gives up (zero before the launch)
    int extra;                   // levels a wait asks for beyond the one it needs (nonzero only to test the timeout)
    long long spin_limit;        // polls of an exchange line before its wait gives up
};

// Shared memory of a CTA with tiles of tx x ty points; co-resident CTAs per SM of that size.
size_t persist2d_smem(int kind, bool ot4, int tx, int ty);
int persist2d_blocks_per_sm(int kind, bool ot4, size_t smem);
// Cooperative launch of nblocks CTAs.
cudaError_t launch_persist2d(int kind, bool ot4, int nblocks, size_t smem, cudaStream_t s, const Persist2D& a);

}  // namespace sa
