// Batched launches for ensembles of independent solvers (host side).
//
// While a plan's `batch` is set, the launchers of the batchable pass kernels do not launch:
// they append a record (the kernel's arguments and its grid) to the batch.  Recording one RK
// step of each solver gives, per solver, the same sequence of kernel families; the ensemble
// then runs position by position, one launch per distinct kernel (template instance and
// shared-memory size) covering the blocks of every solver that uses it.  The batched kernels
// (kernels.cuh, fused_kernels.cuh: *_batch) map their flat block index to (solver, block) through
// the records' block offsets and run the same kernel body as the single launches, so each
// solver's arithmetic is unchanged.
#pragma once

#include <cuda_runtime.h>

#include <cstring>
#include <vector>

namespace sg {

// first member of every record: where the instance's blocks start in the batched grid, and the
// instance's own grid
struct BatchGrid {
    int block0, nbx, nby, nbz;
};

// setup_only: set the kernel's shared-memory limit and return (done before stream capture)
typedef void (*BatchLaunchFn)(const void *recs, int n, int blocks, size_t smem, cudaStream_t s, bool setup_only);

struct BatchEntry {
    const void *key;                 // the batched kernel: entries with the same key and smem share a launch
    size_t smem;                     // dynamic shared memory of one block
    int blocks;                      // blocks of this instance's launch
    std::vector<unsigned char> rec;  // the record (BatchGrid first)
    BatchLaunchFn launch;
    const char *name;
    double bytes;                    // algorithmic bytes of this instance's launch
};

struct Batch {
    std::vector<BatchEntry> entries;  // in launch order
    const char *unbatchable = nullptr;  // name of a launch that had no batched form
};

template <class Rec, class Kern>
void batch_launch_impl(Kern kern, const void *recs, int n, int blocks, size_t smem, int threads, cudaStream_t s,
                       bool setup_only) {
    if (setup_only) {  // always: the kernel's static shared memory counts against the default 48 KB too
        cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        return;
    }
    kern<<<blocks, threads, smem, s>>>((const Rec *)recs, n);
}

template <class Rec>
void batch_add(Batch &b, const Rec &r, const void *key, BatchLaunchFn fn, size_t smem, const char *name, double bytes) {
    BatchEntry e;
    e.key = key;
    e.smem = smem;
    e.blocks = r.grid.nbx * r.grid.nby * r.grid.nbz;
    e.rec.resize(sizeof(Rec));
    std::memcpy(e.rec.data(), &r, sizeof(Rec));
    e.launch = fn;
    e.name = name;
    e.bytes = bytes;
    b.entries.push_back(std::move(e));
}

}  // namespace sg
