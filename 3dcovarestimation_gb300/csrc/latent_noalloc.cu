// Allocation-free variant of the per-image latent-MAP solve (cov3d_gram + cov3d_cost_solve).
//
// Some callers cannot let a library allocate device memory: an application that hands the
// whole GPU to its own memory pool at start-up, a service that must keep every call free of
// cudaMalloc's implicit device synchronisation, or a host program whose allocation budget is
// fixed.  This entry point takes only the caller's inputs and outputs; its intermediate
// per-image Gram matrices, projected images and failure flag live in one file-scope device
// array that every GPU which loads the library holds until the process exits.
#include <mutex>

#include "cov3d_device.cuh"

namespace cov3d {

namespace {

constexpr size_t kScratchBytes = size_t(4) << 20;  // 4 MiB, shared by all calls
static __device__ __align__(256) unsigned char g_latent_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
void *g_scratch_addr[kMaxDevices] = {};

// Device address of the scratch array on the current device, looked up once per device.
int scratch_address(void **out) {
  int dev = 0;
  COV3D_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) {
    set_error("device ordinal %d out of range", dev);
    return COV3D_EINVAL;
  }
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (!g_scratch_addr[dev]) {
    void *ptr = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&ptr, g_latent_scratch);
    if (e != cudaSuccess) return check_cuda(e, "cudaGetSymbolAddress(latent scratch)");
    g_scratch_addr[dev] = ptr;
  }
  *out = g_scratch_addr[dev];
  return COV3D_OK;
}

inline size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

}  // namespace

size_t latent_noalloc_bytes(int n_images, int r) {
  const size_t B = (size_t)n_images, R = (size_t)r;
  return align256(B * R * R * 8) + align256(B * R * 8) + align256(B * 4) + 256;
}

}  // namespace cov3d

using namespace cov3d;

extern "C" int cov3d_latent_map_noalloc(void *stream, int n_images, int P, int r, const void *d_q, int64_t img_stride,
                                        int64_t point_stride, int64_t chan_stride, const void *d_images,
                                        double noise_var, const double *d_linv, void *d_z, void *d_m, int *d_bad) {
  if (n_images < 1 || P < 1 || r < 1 || r > 32 || !d_q || !d_images || !(noise_var > 0.0) || (!d_z && !d_m)) {
    set_error("invalid latent_map_noalloc arguments");
    return COV3D_EINVAL;
  }
  const size_t need = latent_noalloc_bytes(n_images, r);
  if (need > kScratchBytes) {
    set_error("latent_map_noalloc: %d images of rank %d need %zu bytes of scratch; the fixed array holds %zu "
              "(at most %zu images of rank %d)",
              n_images, r, need, kScratchBytes,
              (kScratchBytes - 1024) / ((size_t)r * r * 8 + (size_t)r * 8 + 4), r);
    return COV3D_EINVAL;
  }
  void *base = nullptr;
  COV3D_TRY(scratch_address(&base));
  unsigned char *s = static_cast<unsigned char *>(base);
  const size_t B = (size_t)n_images, R = (size_t)r;
  void *gram = s;
  void *h = s + align256(B * R * R * 8);
  float *yy = reinterpret_cast<float *>(s + align256(B * R * R * 8) + align256(B * R * 8));
  int *bad = reinterpret_cast<int *>(s + align256(B * R * R * 8) + align256(B * R * 8) + align256(B * 4));
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  // the failure flag is the only scratch value that must start at zero; everything else is
  // overwritten by the Gram kernel before it is read
  COV3D_CUDA(cudaMemsetAsync(bad, 0, sizeof(int), st));
  COV3D_TRY(launch_gram(st, n_images, P, r, d_q, img_stride, point_stride, chan_stride, d_images, gram, h, yy));
  COV3D_TRY(launch_solve(st, n_images, r, 0, gram, h, noise_var, d_linv, 1.0, 1.0, nullptr, nullptr, nullptr, nullptr,
                         d_z, d_m, bad));
  if (d_bad) COV3D_CUDA(cudaMemcpyAsync(d_bad, bad, sizeof(int), cudaMemcpyDeviceToDevice, st));
  return COV3D_OK;
}
