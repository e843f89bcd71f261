// devmem.h -- device and pinned-host memory for jobs, without device-wide
// synchronisation.
//
// cudaFree waits for the whole device, so a job that ends with cudaFree
// stalls every other job in flight (serving) and each call of the library
// paid for its allocations again.  Jobs instead take device memory from a
// library-owned, stream-ordered memory pool per device (cudaMallocFromPoolAsync
// / cudaFreeAsync on the job's stream): a free is ordered after the job's own
// work only, and freed blocks stay in the pool for the next job up to a
// retained size (GSDR_POOL_KEEP_MB, default 16384 MiB) instead of going back
// to the driver.  The small pinned host words a job reads back every graph
// launch come from a process-wide free list of pinned slots instead of one
// cudaMallocHost / cudaFreeHost pair per job.
#pragma once
#include <cuda_runtime.h>

#include <cstddef>

namespace gsdr {

// Device memory on the current device, ordered on stream s.
cudaError_t dev_alloc(void** p, size_t bytes, cudaStream_t s);
// Returns p (from dev_alloc on the same device) to the pool after the work
// queued on s so far; p == nullptr is a no-op.
void dev_free(void* p, cudaStream_t s);

// A pinned host block of at most kPinnedSlot bytes (zeroed); nullptr when
// pinned memory cannot be had.
constexpr size_t kPinnedSlot = 1024;
void* pinned_slot();
void pinned_release(void* p);

// A pinned host buffer of at least `bytes`, owned by the calling thread and
// reused by its later calls (grown when a call needs more; released when the
// thread ends).  Its contents last until the thread's next call.  nullptr when
// pinned memory cannot be had.
void* pinned_scratch(size_t bytes);

}  // namespace gsdr
