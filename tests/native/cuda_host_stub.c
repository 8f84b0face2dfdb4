/* Host-memory stand-ins for the CUDA runtime calls that libgbp's serving loop makes itself (pinned buffers, the
 * device ordinal, the free-memory query), so that the loop's host logic (tickets, batching, admission, borrowed
 * instance arrays, shutdown) builds and runs on a machine without a GPU against the oracle test double
 * tests/plugin/gbp_oracle_shim.c.  Test infrastructure only: libgbp itself links the CUDA runtime. */
#include <stdlib.h>

#include <cuda_runtime_api.h>

cudaError_t cudaMallocHost(void** ptr, size_t size)
{
   *ptr = malloc(size > 0 ? size : 1);
   return *ptr != NULL ? cudaSuccess : cudaErrorMemoryAllocation;
}

/* the C++ overloads of cudaMallocHost in cuda_runtime.h allocate through this one */
cudaError_t cudaHostAlloc(void** ptr, size_t size, unsigned int flags)
{
   (void)flags;
   return cudaMallocHost(ptr, size);
}

cudaError_t cudaFreeHost(void* ptr)
{
   free(ptr);
   return cudaSuccess;
}

cudaError_t cudaSetDevice(int device)
{
   return device == 0 ? cudaSuccess : cudaErrorInvalidDevice;
}

cudaError_t cudaMemGetInfo(size_t* freemem, size_t* total)
{
   *freemem = (size_t)64 << 30;
   *total = (size_t)96 << 30;
   return cudaSuccess;
}
