// tc_noalloc.cu — tc_blas_setup_insertion_noalloc: the blas_setup_insertion
// stage for callers that cannot allocate device memory.
//
// Who needs it: a host application that owns every byte of device memory
// itself (a renderer whose buffers come from one pre-sized pool or are
// imported from another API's allocations) cannot let a library call
// cudaMalloc behind its back, and a real-time frame loop cannot afford the
// implicit device synchronisation cudaMalloc/cudaFree may perform. Such a
// caller also cannot create a tc_context, which allocates its scratch. This
// entry point takes no context: the caller passes the frame's own buffers
// (SceneBuilding, Readback), and the stage's look-back scratch lives in a
// fixed file-scope __device__ array of this library.
//
// The array (g_blasSetupScratch) is sized for TC_NOALLOC_MAX_INSTANCES
// instances (4096 tiles of 256: 32 KiB of look-back state plus 256 bytes of
// counters). Every GPU that loads the library holds it until the process
// exits. All calls on a device share it and it keeps the last call's
// contents: each call clears the whole array (one 33,024-byte cudaMemsetAsync
// on the caller's stream) before its launch. Calls that overlap on the GPU (two
// streams, or two host threads with unordered streams) race on it.
//
// Set-up: every call looks the array's device address up with
// cudaGetSymbolAddress in the caller's current context (the device that is
// current at the call) and passes that pointer to the kernel; nothing is
// cached, so a context created after cudaDeviceReset, or a caller that makes
// its own context current, gets the address in that context. The first call
// in a context may load the library's device code (lazy module loading):
// make it before any stream capture. In host code the name g_blasSetupScratch
// is only a host-side stand-in for the symbol, never a device address.
#include <algorithm>
#include <cstring>

#include "tc_kernels.h"
#include "tc_stage.cuh"

namespace tc {

namespace {

constexpr u32    kNoAllocTiles = TC_NOALLOC_MAX_INSTANCES / kInstanceTile;
constexpr size_t kCounterBytes = 256;  // ticket u32 @0, done u32 @4, total u64 @8, error word u32 @16
constexpr size_t kNoAllocBytes = kCounterBytes + (size_t)kNoAllocTiles * sizeof(u64);
static_assert(TC_NOALLOC_MAX_INSTANCES % kInstanceTile == 0, "whole tiles");

static __device__ __align__(256) unsigned char g_blasSetupScratch[kNoAllocBytes];

// Device address of g_blasSetupScratch in the current context.
tc_status scratch_address(unsigned char** out)
{
  void* address = nullptr;
  if(cudaGetSymbolAddress(&address, g_blasSetupScratch) != cudaSuccess || address == nullptr)
    return TC_ERR_CUDA;
  *out = static_cast<unsigned char*>(address);
  return TC_OK;
}

}  // namespace

}  // namespace tc

using namespace tc;

extern "C" tc_status tc_blas_setup_insertion_noalloc(const tc_frame_args* a, uint32_t* deviceErrors, void* stream)
{
  if(!a || !a->build || !a->readback)
    return TC_ERR_INVALID_ARG;
  if(a->numInstances > TC_NOALLOC_MAX_INSTANCES)
    return TC_ERR_CAPACITY;
  unsigned char* scratch = nullptr;
  tc_status      st      = scratch_address(&scratch);
  if(st != TC_OK)
    return st;
  cudaStream_t s     = reinterpret_cast<cudaStream_t>(stream);
  const u32    tiles = std::max(1u, (a->numInstances + kInstanceTile - 1) / kInstanceTile);
  // counters and look-back states start at zero; the kernel sizes its tiles
  // from SceneBuilding.numRenderInstances, so all of them are cleared
  if(cudaMemsetAsync(scratch, 0, kNoAllocBytes, s) != cudaSuccess)
    return TC_ERR_CUDA;

  StageCtx c;
  std::memset(&c, 0, sizeof(c));
  c.build                = reinterpret_cast<tc_SceneBuilding*>(a->build);
  c.readback             = reinterpret_cast<tc_Readback*>(a->readback);
  c.numInstances         = a->numInstances;
  c.instEnd              = a->numInstances;
  c.fuseSetup            = kNoSetup;
  c.run                  = kAllRuns;
  c.errorWord            = deviceErrors ? deviceErrors : reinterpret_cast<u32*>(scratch + 16);
  c.scratch.ticket       = reinterpret_cast<u32*>(scratch + 0);
  c.scratch.done         = reinterpret_cast<u32*>(scratch + 4);
  c.scratch.totals       = reinterpret_cast<u64*>(scratch + 8);
  c.scratch.lbState      = reinterpret_cast<u64*>(scratch + kCounterBytes);
  c.scratch.lbStride     = kNoAllocTiles;
  c.scratch.selfClean    = 0;  // cleared by the memset above
  c.scratch.itemCapacity = TC_NOALLOC_MAX_INSTANCES;
  c.spinLimit            = kSpinLimit;
  if(launch_blas_setup_insertion(c, tiles, kInstanceTile, s) != cudaSuccess)
    return TC_ERR_CUDA;
  return TC_OK;
}
