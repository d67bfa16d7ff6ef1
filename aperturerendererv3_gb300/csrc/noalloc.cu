// ar_render_noalloc: the path tracer for callers that must not allocate device
// memory.
//
// Who needs it: code that renders inside a frame loop or a memory-pool regime
// where cudaMalloc / cudaFree are off limits -- cudaFree synchronises the whole
// device, a pool-managed application forbids raw allocations, and an embedding
// host may own all device memory itself.  ar_render keeps its wavefront working
// set (path state, queues, shadow rays: ~190 bytes per path in flight) in
// buffers it allocates on first use; this entry point instead runs every wave
// out of one fixed scratch array that lives in the library image.
//
// The scratch array is a file-scope __device__ array of AR_NOALLOC_SCRATCH_BYTES
// (8 MiB).  Every GPU that loads the library holds it until the process exits.
// Its device address is looked up once per device with cudaGetSymbolAddress, on
// the first call made with that device current; make that first call before
// any stream capture begins.  The address is kept for the life of the process:
// cudaDeviceReset unloads the module (and ends every context of the device), so
// no call may follow a reset of that device.  All calls share the array and it keeps the last
// call's contents: each call re-initialises what must start fresh (queue
// counters, the caller's output) before use.  Calls whose work overlaps on the
// GPU (other streams, other host threads) race on the array; serialise them.
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/aperture/ar.h"
#include "ar_internal.h"

struct ar_ctx
{
    ar::Ctx c;
};

#define AR_NOALLOC_MAX_DEVICES 64

static __device__ __align__(256) unsigned char g_noalloc_scratch[AR_NOALLOC_SCRATCH_BYTES];

namespace
{
using namespace ar;

// bytes per path of the wavefront working set (one entry of each array)
constexpr size_t kPathBytes = sizeof(uint64_t) + 2 * sizeof(uint32_t) + 2 * sizeof(float4) + 2 * sizeof(float) +
                              2 * sizeof(uint32_t) + sizeof(float4) + sizeof(int) + sizeof(float4) + sizeof(float) +
                              sizeof(int) + 3 * sizeof(float) + sizeof(int) + 2 * sizeof(float4) + sizeof(float) +
                              sizeof(uint8_t) + sizeof(float) + 2 * sizeof(int) + sizeof(float4) + sizeof(int) +
                              sizeof(int) + sizeof(int2);
constexpr int kArrays = 27;
constexpr size_t kAlign = 256;
// largest wave that fits the scratch array (array starts padded to 256 bytes)
constexpr int kMaxPaths = (int)(((AR_NOALLOC_SCRATCH_BYTES - kAlign * (kArrays + 1)) / kPathBytes) & ~255u);

std::mutex g_mu;
unsigned char* g_scratch_ptr[AR_NOALLOC_MAX_DEVICES] = {};

cudaError_t scratch_for_device(int dev, unsigned char** out)
{
    if (dev < 0 || dev >= AR_NOALLOC_MAX_DEVICES) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> g(g_mu);
    if (!g_scratch_ptr[dev])
    {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);  // device `dev` is current here
        if (e != cudaSuccess) return e;
        g_scratch_ptr[dev] = static_cast<unsigned char*>(p);
    }
    *out = g_scratch_ptr[dev];
    return cudaSuccess;
}

template <typename T>
T* carve(unsigned char*& cur, size_t n)
{
    T* p = reinterpret_cast<T*>(cur);
    cur += ((n * sizeof(T) + kAlign - 1) / kAlign) * kAlign;
    return p;
}

} // namespace

extern "C" ar_status ar_render_noalloc(ar_ctx* ctx, const ar_render_params* prm, double* out_xyz_device, void* stream)
{
    if (!ctx || !prm || !out_xyz_device) return AR_ERR_INVALID;
    Ctx& c = ctx->c;
    if (!c.built)
    {
        c.last_error = "render before ar_scene_build";
        return AR_ERR_STATE;
    }
    if (prm->width <= 0 || prm->height <= 0 || prm->spp <= 0 || prm->max_depth <= 0 || prm->max_depth > 0xffff)
    {
        c.last_error = "render_noalloc: bad resolution, spp or depth";
        return AR_ERR_INVALID;
    }
    if ((long long)prm->width * prm->height > 0x7fffffffll)
    {
        c.last_error = "render_noalloc: more than 2^31 - 1 pixels";  // pixel indices are 32-bit
        return AR_ERR_INVALID;
    }
    if (prm->wave_paths > kMaxPaths)
    {
        c.last_error = "render_noalloc: wave_paths " + std::to_string(prm->wave_paths) + " exceeds the scratch limit of " +
                       std::to_string(kMaxPaths) + " paths (" + std::to_string(AR_NOALLOC_SCRATCH_BYTES) + " bytes)";
        return AR_ERR_INVALID;
    }
    if (prm->profile || prm->guide || prm->denoise_record)
    {
        c.last_error = "render_noalloc: profiling, path guiding and denoiser records need allocations; use ar_render";
        return AR_ERR_INVALID;
    }
    cudaError_t e = cudaSetDevice(c.device);
    unsigned char* base = nullptr;
    if (e == cudaSuccess) e = scratch_for_device(c.device, &base);
    if (e != cudaSuccess)
    {
        c.last_error = std::string("render_noalloc setup: ") + cudaGetErrorString(e);
        return AR_ERR_CUDA;
    }
    const int cap = prm->wave_paths > 0 ? prm->wave_paths : kMaxPaths;
    WaveBuffers wb{};
    unsigned char* cur = base;
    const size_t n = (size_t)cap;
    wb.ps.rng = carve<uint64_t>(cur, n);
    wb.ps.pixel = carve<uint32_t>(cur, n);
    wb.ps.frame = carve<uint32_t>(cur, n);
    wb.ps.ray_o = carve<float4>(cur, n);
    wb.ps.ray_d = carve<float4>(cur, n);
    wb.ps.radiance = carve<float>(cur, n);
    wb.ps.mask = carve<float>(cur, n);
    wb.ps.depths = carve<uint32_t>(cur, n);
    wb.ps.flags = carve<uint32_t>(cur, n);
    wb.ps.media_v = carve<float4>(cur, n);
    wb.ps.media_depth = carve<int>(cur, n);
    wb.ps.prev = carve<float4>(cur, n);
    wb.ps.hit_t = carve<float>(cur, n);
    wb.ps.hit_slot = carve<int>(cur, n);
    wb.ps.q_slot = carve<int>(cur, n);
    wb.ps.hit_nrm = carve<float4>(cur, n);
    wb.ps.out_xyz = carve<float>(cur, 3 * n);
    wb.ps.capacity = cap;
    wb.sq.path = carve<int>(cur, n);
    wb.sq.o = carve<float4>(cur, n);
    wb.sq.d = carve<float4>(cur, n);
    wb.sq.v_occ = carve<float>(cur, n);
    wb.sq.valid_unocc = carve<uint8_t>(cur, n);
    wb.sq.sdf_eps = carve<float>(cur, n);
    wb.queue[0] = carve<int>(cur, n);
    wb.queue[1] = carve<int>(cur, n);
    wb.pq = carve<int2>(cur, n);
    wb.counters = carve<int>(cur, AR_CNT_COUNT);
    wb.pend_list = carve<int>(cur, n);
    if ((size_t)(cur - base) > AR_NOALLOC_SCRATCH_BYTES)
    {
        c.last_error = "render_noalloc: scratch layout exceeds the array";
        return AR_ERR_INVALID;
    }
    wb.accum = out_xyz_device;
    wb.stream = stream ? (cudaStream_t)stream : c.stream;

    RenderLaunch rl{};
    rl.width = prm->width;
    rl.height = prm->height;
    rl.spp = prm->spp;
    rl.max_depth = prm->max_depth;
    for (int k = 0; k < 3; ++k)
    {
        rl.cam_o[k] = prm->cam_origin[k];
        rl.cam_d[k] = prm->cam_dir[k];
    }
    rl.fov_deg = prm->fov_deg;
    rl.use_nee = prm->use_nee;
    rl.seed = prm->seed;
    rl.first_frame = prm->first_frame;
    rl.profile = 0;
    rl.sample_block = std::min(AR_SAMPLE_BLOCK, std::max(1, rl.spp));  // the path order of ar_render
    // the same test as ar_render's (SDF objects evaluate their field; no allocation)
    const int camera_inside = camera_inside_any(c, rl.cam_o);
    DevScene sc = dev_scene(c);
    sc.stats = nullptr;
    sc.camera_inside = camera_inside;
    const long long npix = (long long)rl.width * rl.height;
    const long long total = npix * rl.spp;
    // work the context queued without waiting (ar_scene_update_texels with a
    // NULL stream, for instance) comes first when the caller passes a stream
    // of its own; the event was created with the context
    if (wb.stream != c.stream)
    {
        e = cudaEventRecord(c.order_event, c.stream);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(wb.stream, c.order_event, 0);
    }
    // the caller's buffer is the FP64 accumulator: clear it first
    if (e == cudaSuccess) e = cudaMemsetAsync(out_xyz_device, 0, (size_t)npix * 3 * sizeof(double), wb.stream);
    for (long long first = 0; first < total && e == cudaSuccess; first += cap)
    {
        const int nw = (int)std::min<long long>(cap, total - first);
        e = launch_render_wave_buffers(sc, wb, c.device, rl, camera_inside, first, nw, c.d_err);
    }
    if (e == cudaSuccess)
    {
        const long long nv = npix * 3;
        launch_scale_means(out_xyz_device, nv, 1.0 / (double)rl.spp, wb.stream);
        e = cudaGetLastError();
    }
    if (e != cudaSuccess)
    {
        c.last_error = std::string("render_noalloc: ") + cudaGetErrorString(e);
        return AR_ERR_CUDA;
    }
    return AR_OK;
}

static_assert(kMaxPaths == AR_NOALLOC_MAX_PATHS, "AR_NOALLOC_MAX_PATHS in ar.h must match the scratch layout");
