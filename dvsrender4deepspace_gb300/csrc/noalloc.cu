// Camera render that allocates nothing.
//
// Some callers cannot call cudaMalloc while they render: a frame loop that
// runs under a fixed, pre-reserved device-memory budget; a host framework
// that owns all device memory through its own pool, where an extra
// allocation escapes its accounting and may fail or fragment the pool; or
// code on a latency-critical path, where cudaMalloc/cudaFree can stall or
// synchronize the device.  dvs_cam_render_noalloc serves them: the scene is
// created beforehand, the caller passes device buffers for the outputs, and
// the only intermediate storage (the pose and the per-pixel FP64 radiance
// and depth in Morton-rank order) is the file-scope array below.
//
// The array is sized for the largest configured sensor, 1280 x 720 pixels
// (about 11 MB), and every GPU that loads the library keeps it until the
// process exits.  It is shared by all calls, so calls that overlap on the
// GPU (different streams or threads at the same time) race on it.  Each call
// overwrites all of it that it reads, so nothing needs clearing between calls.
// Creating the scene does the per-device set-up (dvsgb_noalloc_prepare):
// it looks up the array's device address with cudaGetSymbolAddress and loads
// the render's kernels, so the render itself loads and reserves nothing.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "dvs_gb300.h"
#include "kernels.h"

using namespace dvsgb;

// Accessors defined in capi.cu.
SceneView dvsgb_scene_view(const dvs_scene *scene);
int dvsgb_scene_device(const dvs_scene *scene);
int dvsgb_set_error(int code, const char *message);

namespace {

constexpr size_t kNoAllocMaxPixels = 1280 * 720;
constexpr size_t kPoseBytes = 256;
constexpr size_t kScratchBytes = kPoseBytes + kNoAllocMaxPixels * (sizeof(double) + sizeof(float));
// layout: the pose, then the FP64 radiance (8-byte aligned), then the depth
static_assert(sizeof(CellPose) <= kPoseBytes && kPoseBytes % alignof(double) == 0, "no-allocation scratch layout");

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

constexpr int kMaxDevices = 128;
std::mutex g_setup_mutex;
void *g_scratch_address[kMaxDevices] = {};  // device address of g_noalloc_scratch, per device
bool g_kernels_loaded[kMaxDevices][4] = {};  // camera kernels loaded, per device and scene geometry

__device__ __forceinline__ float3 normalize3(float3 v) {
  float len = sqrtf(v.x * v.x + v.y * v.y + v.z * v.z);
  if (len > 0.0f) return make_float3(v.x / len, v.y / len, v.z / len);
  return make_float3(0.0f, 0.0f, 0.0f);
}

// The pose used as given (as dvs_cam_render does): quaternion unchanged, light normalized.
__global__ void noalloc_pose_kernel(dvs_optical_state s, CellPose *out) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const float3 ln = normalize3(make_float3(s.light.x, s.light.y, s.light.z));
  CellPose o;
  o.px = s.position.x; o.py = s.position.y; o.pz = s.position.z; o.intensity = s.intensity;
  o.qx = s.rotation.x; o.qy = s.rotation.y; o.qz = s.rotation.z; o.qw = s.rotation.w;
  o.lx = ln.x; o.ly = ln.y; o.lz = ln.z; o.pad = 0;
  *out = o;
}

// Once per device, with that device current: the device address of the array.
int scratch_for_device(int device, unsigned char **out) {
  if (device < 0 || device >= kMaxDevices) return dvsgb_set_error(DVS_ERR_INVALID, "device ordinal out of range");
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (!g_scratch_address[device]) {
    void *ptr = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
    if (e != cudaSuccess || !ptr)
      return dvsgb_set_error(DVS_ERR_CUDA, (std::string("[CUDA Error] in no-allocation scratch address : ") +
                                            cudaGetErrorString(e)).c_str());
    g_scratch_address[device] = ptr;
  }
  *out = static_cast<unsigned char *>(g_scratch_address[device]);
  return DVS_OK;
}

}  // namespace

// Set-up of the no-allocation render, called by dvs_scene_create and
// dvs_scene_view_create with the scene's device current.  Under CUDA's lazy
// module loading the first use of a module or kernel is what loads it, and
// loading the module that holds the static array reserves the array's device
// memory.  Doing that here, where the caller is creating a scene and may
// allocate, leaves nothing to load or reserve in the render itself: the
// array's address is looked up and every kernel the render launches for
// this geometry is loaded.
int dvsgb_noalloc_prepare(int device, int geometry) {
  unsigned char *base = nullptr;
  int status = scratch_for_device(device, &base);
  if (status != DVS_OK) return status;
  const int g = geometry & 3;
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (g_kernels_loaded[device][g]) return DVS_OK;
  cudaFuncAttributes attr;
  cudaError_t e = cudaFuncGetAttributes(&attr, noalloc_pose_kernel);
  if (e == cudaSuccess) e = preload_camera_kernels(g);
  if (e != cudaSuccess)
    return dvsgb_set_error(DVS_ERR_CUDA, (std::string("[CUDA Error] in no-allocation kernel set-up : ") +
                                          cudaGetErrorString(e)).c_str());
  g_kernels_loaded[device][g] = true;
  return DVS_OK;
}

extern "C" int dvs_cam_render_noalloc(dvs_scene *scene, const dvs_optical_state *pose, float *radiance, float *depth,
                                      void *stream) {
  if (!scene || !pose || !radiance) return dvsgb_set_error(DVS_ERR_INVALID, "invalid parallel optical request");
  const SceneView view = dvsgb_scene_view(scene);
  const size_t n = size_t(view.width) * size_t(view.height);
  if (n > kNoAllocMaxPixels)
    return dvsgb_set_error(DVS_ERR_INVALID,
                           ("image of " + std::to_string(n) + " pixels exceeds the no-allocation scratch limit of " +
                            std::to_string(kNoAllocMaxPixels) + " pixels (1280x720)").c_str());
  int previous = 0;
  if (cudaGetDevice(&previous) != cudaSuccess) return dvsgb_set_error(DVS_ERR_CUDA, "[CUDA Error] in get device");
  const int device = dvsgb_scene_device(scene);
  if (device != previous && cudaSetDevice(device) != cudaSuccess)
    return dvsgb_set_error(DVS_ERR_CUDA, "[CUDA Error] in select scene device");
  int status = DVS_OK;
  unsigned char *base = nullptr;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if ((status = scratch_for_device(device, &base)) == DVS_OK) {
    CellPose *d_pose = reinterpret_cast<CellPose *>(base);
    double *d_radiance = reinterpret_cast<double *>(base + kPoseBytes);
    float *d_depth = reinterpret_cast<float *>(base + kPoseBytes + kNoAllocMaxPixels * sizeof(double));
    noalloc_pose_kernel<<<1, 32, 0, s>>>(*pose, d_pose);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = launch_trace_cells(view, (int)n, d_pose, 0, 1, 0, d_radiance, d_depth, nullptr, s);
    if (e == cudaSuccess)
      e = launch_radiance_to_float((int)n, view.pixel_of_rank, d_radiance, d_depth, radiance, depth, s);
    if (e != cudaSuccess)
      status = dvsgb_set_error(DVS_ERR_CUDA, (std::string("[CUDA Error] in no-allocation camera render : ") +
                                              cudaGetErrorString(e)).c_str());
  }
  if (device != previous) cudaSetDevice(previous);
  return status;
}
