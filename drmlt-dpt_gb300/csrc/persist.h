// Host side of the persistent chain-loop schedule (persist.cu).
#pragma once
#include <cuda_runtime.h>

namespace drmlt {

struct RunParams;
struct PathRec;

// Error bits of the persistent schedule's status word.
enum : int {
    kPersistIdleLane = 1,   // a lane worker saw no progress for the wait limit
    kPersistIdleTeam = 2,   // a team worker saw no progress for the wait limit
    kPersistCellWait = 4,   // a queue cell was not handed over within the wait limit
    kPersistBadPhase = 8    // a chain came back in a phase the lane workers do not run
};

// Device buffers of the persistent schedule (owned by the renderer).
struct PersistBuffers {
    void *laneCells, *teamCells;      // queue cells (16 B each), N per queue
    unsigned long long *ctl;          // lane head, lane tail, team head, team tail, progress, done
    int *status;
    int *chainIter, *chainPhase;      // per chain
    PathRec *ystar;                   // per chain: Green's reverse path record
    float *rows;                      // per worker block: gradient + Hessian rows
    int rowBlocks;                    // blocks the rows are sized for
};

// Resident blocks per SM of the persistent kernel (128 threads, smem bytes of
// dynamic shared memory), and the kernel's register count.
int persist_blocks_per_sm(size_t smem, int *regs);

// Runs every chain from its current iteration `begin` to min(end, its samples)
// in one cooperative launch of `grid` blocks on `stream`: SMs [0, teamSms)
// run the derivative / Gaussian workers, the others the path-tracing lane
// workers. waitLimit: idle polls without progress before a worker gives up.
cudaError_t persist_run(const RunParams &p, const PersistBuffers &b, long long begin, long long end, int grid,
                        int teamSms, long long waitLimit, size_t smem, cudaStream_t stream);

}  // namespace drmlt
