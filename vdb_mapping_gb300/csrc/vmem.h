// Device arrays that grow in place: a virtual address range reserved once,
// backed on demand by physical chunks (CUDA virtual memory management). A
// leaf or block slot therefore keeps its address for the life of the map, and
// growing a pool maps more memory behind the same pointer instead of
// allocating a larger array and copying the old one into it.
//
// The driver's entry points are looked up through the runtime
// (cudaGetDriverEntryPointByVersion), so the library links only cudart and
// loads on machines without a driver (it then reports VDBG_ERR_CUDA on use).
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <mutex>
#include <utility>
#include <vector>

namespace vmem {

struct Api
{
  decltype(&cuMemAddressReserve) reserve               = nullptr;
  decltype(&cuMemAddressFree) address_free             = nullptr;
  decltype(&cuMemCreate) create                        = nullptr;
  decltype(&cuMemRelease) release                      = nullptr;
  decltype(&cuMemMap) map                              = nullptr;
  decltype(&cuMemUnmap) unmap                          = nullptr;
  decltype(&cuMemSetAccess) set_access                 = nullptr;
  decltype(&cuMemGetAllocationGranularity) granularity = nullptr;
  bool ok                                              = false;
};

// The entry points, looked up once per process; nullptr when the driver does
// not provide them.
inline const Api* api()
{
  static Api a;
  static std::once_flag once;
  std::call_once(once, [] {
    auto get = [](const char* name, void** fn) {
      cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
      const cudaError_t e = cudaGetDriverEntryPointByVersion(name, fn, 12000, cudaEnableDefault, &q);
      return e == cudaSuccess && q == cudaDriverEntryPointSuccess && *fn != nullptr;
    };
    a.ok = get("cuMemAddressReserve", reinterpret_cast<void**>(&a.reserve)) &&
           get("cuMemAddressFree", reinterpret_cast<void**>(&a.address_free)) &&
           get("cuMemCreate", reinterpret_cast<void**>(&a.create)) &&
           get("cuMemRelease", reinterpret_cast<void**>(&a.release)) &&
           get("cuMemMap", reinterpret_cast<void**>(&a.map)) &&
           get("cuMemUnmap", reinterpret_cast<void**>(&a.unmap)) &&
           get("cuMemSetAccess", reinterpret_cast<void**>(&a.set_access)) &&
           get("cuMemGetAllocationGranularity", reinterpret_cast<void**>(&a.granularity));
    cudaGetLastError();
  });
  return a.ok ? &a : nullptr;
}

inline CUmemAllocationProp device_prop(int device)
{
  CUmemAllocationProp p{};
  p.type          = CU_MEM_ALLOCATION_TYPE_PINNED;
  p.location.type = CU_MEM_LOCATION_TYPE_DEVICE;
  p.location.id   = device;
  return p;
}

// Physical page size of device allocations on `device` (2 MiB on GB300).
inline size_t granularity(int device)
{
  const Api* v = api();
  if (!v) return 0;
  const CUmemAllocationProp p = device_prop(device);
  size_t g                    = 0;
  if (v->granularity(&g, &p, CU_MEM_ALLOC_GRANULARITY_MINIMUM) != CUDA_SUCCESS) return 0;
  return g;
}

inline size_t round_up(size_t b, size_t g) { return (b + g - 1) / g * g; }

// One growable array. `base` never changes once reserved.
struct Array
{
  char* base      = nullptr;
  size_t reserved = 0;  // virtual bytes
  size_t mapped   = 0;  // bytes backed by physical memory, from base
  std::vector<std::pair<CUmemGenericAllocationHandle, size_t>> chunks;  // in address order
};

enum class Status
{
  ok,
  no_driver,
  out_of_memory,
  failed
};

// Reserves up to `want` bytes of address space (at least `need`): large
// reservations are retried at half the size until one succeeds.
inline Status reserve(Array& a, size_t need, size_t want, size_t gran)
{
  const Api* v = api();
  if (!v || gran == 0) return Status::no_driver;
  need = round_up(need > 0 ? need : gran, gran);
  want = round_up(want > need ? want : need, gran);
  for (size_t r = want;; r = round_up(r / 2, gran))
  {
    if (r < need) r = need;
    CUdeviceptr p = 0;
    if (v->reserve(&p, r, gran, 0, 0) == CUDA_SUCCESS)
    {
      a.base     = reinterpret_cast<char*>(p);
      a.reserved = r;
      a.mapped   = 0;
      return Status::ok;
    }
    if (r == need) return Status::out_of_memory;
  }
}

// Backs [0, bytes) (rounded up to the page size) with physical memory on
// `device`; *added receives the bytes newly mapped.
inline Status commit(Array& a, size_t bytes, size_t gran, int device, size_t* added)
{
  *added       = 0;
  const Api* v = api();
  if (!v) return Status::no_driver;
  bytes = round_up(bytes, gran);
  if (bytes <= a.mapped) return Status::ok;
  if (bytes > a.reserved) return Status::out_of_memory;
  const size_t n                 = bytes - a.mapped;
  const CUmemAllocationProp prop = device_prop(device);
  CUmemGenericAllocationHandle h = 0;
  CUresult r                     = v->create(&h, n, &prop, 0);
  if (r != CUDA_SUCCESS) return r == CUDA_ERROR_OUT_OF_MEMORY ? Status::out_of_memory : Status::failed;
  const CUdeviceptr at = reinterpret_cast<CUdeviceptr>(a.base) + a.mapped;
  r                    = v->map(at, n, 0, h, 0);
  if (r != CUDA_SUCCESS)
  {
    v->release(h);
    return Status::failed;
  }
  CUmemAccessDesc acc{};
  acc.location.type = CU_MEM_LOCATION_TYPE_DEVICE;
  acc.location.id   = device;
  acc.flags         = CU_MEM_ACCESS_FLAGS_PROT_READWRITE;
  r                 = v->set_access(at, n, &acc, 1);
  if (r != CUDA_SUCCESS)
  {
    v->unmap(at, n);
    v->release(h);
    return Status::failed;
  }
  a.chunks.emplace_back(h, n);
  a.mapped += n;
  *added = n;
  return Status::ok;
}

// Unmaps and releases everything and frees the address range. The caller has
// made sure no work on the device still uses the array.
inline void release(Array& a)
{
  const Api* v = api();
  if (v && a.base)
  {
    size_t off = 0;
    for (auto& c : a.chunks)
    {
      v->unmap(reinterpret_cast<CUdeviceptr>(a.base) + off, c.second);
      v->release(c.first);
      off += c.second;
    }
    v->address_free(reinterpret_cast<CUdeviceptr>(a.base), a.reserved);
  }
  a = Array{};
}

} // namespace vmem
