// noalloc.cu -- the material-point update (J2.update, J2.java:163-296) for callers that must
// not allocate device memory.
//
// nf_material_point_update stages its inputs in buffers it obtains with cudaMalloc and
// releases with cudaFree. Some callers cannot accept that: cudaMalloc and cudaFree
// synchronise the whole device, which stalls a caller that keeps other streams busy; and a
// host application whose device memory is owned by its own pool allocator (a JVM-side or
// framework arena that has reserved the GPU's memory budget) has none left to hand out. This
// variant stages through one file-scope device array instead, so a call performs only copies
// and a kernel launch.
//
// The array holds NF_NOALLOC_MAX_POINTS points (27 doubles each, 1.77 MB) and lives on every
// GPU that loads this library until the process exits. The first call on each device, with
// that device current, looks the array's device address up (cudaGetSymbolAddress) and creates
// the library's own non-blocking stream for that device; make that first call before any
// stream capture begins. Every later call copies in, runs the kernel and copies out on that
// stream, then waits for that stream alone: a non-blocking stream has no implicit ordering
// with the legacy default stream or with the caller's other streams, so the call neither waits
// for nor holds up the caller's other work. All calls share the array: a call overwrites every
// staging slot it reads before the kernel runs, so nothing stale is used, but calls made from
// several host threads at once race on it.
#include "nf_internal.h"

#include <mutex>

namespace nf {
const char *validate_material(const nf_material &m);
MatDev material_constants(const nf_material &m, int formulation);
void set_thread_error(const char *message);
}  // namespace nf

using namespace nf;

namespace {

constexpr int NF_NOALLOC_MAX_POINTS = 8192;
constexpr int STAGE_DOUBLES = 27;      // sig 4, back 4, eps 1, work 1, strain 4, dgamma 1,
                                       // damage: failure, fracture energy, E, geometry 5,
                                       // strength, softening, width
constexpr int MAX_DEVICES = 64;

static __device__ __align__(256) double g_point_stage[(size_t)NF_NOALLOC_MAX_POINTS * STAGE_DOUBLES];

std::mutex g_stage_lock;
double *g_stage_address[MAX_DEVICES] = {nullptr};
cudaStream_t g_stage_stream[MAX_DEVICES] = {nullptr};

nf_status stage_error(nf_status st, const char *msg) {
    set_thread_error(msg);
    return st;
}

nf_status stage_cuda_error(const char *what, cudaError_t e) {
    (void)cudaGetLastError();                  // leave no error behind for a later call
    char buf[256];
    snprintf(buf, sizeof buf, "%s: %s", what, cudaGetErrorString(e));
    return stage_error(NF_EDEVICE, buf);
}

// Device address of the staging array and the library's stream on the current device, set up
// on first use.
nf_status stage_for_current_device(double **out, cudaStream_t *stream) {
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= MAX_DEVICES)
        return stage_error(NF_EDEVICE, "no usable current CUDA device");
    std::lock_guard<std::mutex> guard(g_stage_lock);
    if (!g_stage_address[dev]) {
        void *p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_point_stage);
        if (e != cudaSuccess || !p)
            return stage_cuda_error("cudaGetSymbolAddress of the staging array failed", e);
        cudaStream_t st = nullptr;
        const cudaError_t es = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
        if (es != cudaSuccess) return stage_cuda_error("creating the staging stream failed", es);
        g_stage_stream[dev] = st;
        g_stage_address[dev] = static_cast<double *>(p);
    }
    *out = g_stage_address[dev];
    *stream = g_stage_stream[dev];
    return NF_OK;
}

cudaError_t put(double *dst, const double *src, size_t count, cudaStream_t st) {
    return cudaMemcpyAsync(dst, src, sizeof(double) * count, cudaMemcpyHostToDevice, st);
}
cudaError_t get(double *dst, const double *src, size_t count, cudaStream_t st) {
    return cudaMemcpyAsync(dst, src, sizeof(double) * count, cudaMemcpyDeviceToHost, st);
}

}  // namespace

extern "C" nf_status nf_material_point_update_static(
        const nf_material *material, int32_t formulation, int32_t count, double *sig,
        double *back, double *eps_p, double *work, const double *strain, double strain_dt,
        const nf_damage_points *damage, double *dgamma) {
    const char *why = validate_material(*material);
    if (why) return stage_error(NF_EINVAL, why);
    if (count <= 0) return NF_OK;
    if (count > NF_NOALLOC_MAX_POINTS) {
        char buf[160];
        snprintf(buf, sizeof buf,
                 "nf_material_point_update_static takes at most %d points per call; got %d",
                 NF_NOALLOC_MAX_POINTS, count);
        return stage_error(NF_EINVAL, buf);
    }
    double *base = nullptr;
    cudaStream_t stream = nullptr;
    nf_status st = stage_for_current_device(&base, &stream);
    if (st) return st;
    const size_t n = (size_t)count;
    const bool dm = damage && damage->failure_strain;
    double *dsig = base, *dback = dsig + 4 * n, *deps = dback + 4 * n, *dwork = deps + n;
    double *dstrain = dwork + n, *dg = dstrain + 4 * n;
    double *fail_ = nullptr, *gf = nullptr, *yo = nullptr, *geom = nullptr, *str = nullptr,
           *soft = nullptr, *wid = nullptr;
    (void)cudaGetLastError();                  // an error left by unrelated earlier work
    cudaError_t e = cudaSuccess;
    auto in = [&](double *dst, const double *src, size_t c) {
        if (e == cudaSuccess) e = put(dst, src, c, stream);
    };
    in(dsig, sig, 4 * n);
    in(dback, back, 4 * n);
    in(deps, eps_p, n);
    in(dwork, work, n);
    in(dstrain, strain, 4 * n);
    if (dm) {
        fail_ = dg + n; gf = fail_ + n; yo = gf + n; geom = yo + n; str = geom + 5 * n;
        soft = str + n; wid = soft + n;
        in(fail_, damage->failure_strain, n);
        in(gf, damage->fracture_energy, n);
        in(yo, damage->youngs_modulus, n);
        in(geom, damage->geometry, 5 * n);
        in(str, damage->strength, n);
        in(soft, damage->softening, n);
        in(wid, damage->width, n);
    }
    if (e != cudaSuccess) {
        (void)cudaStreamSynchronize(stream);
        return stage_cuda_error("copy into the staging array failed", e);
    }
    launch_material_points(material_constants(*material, formulation), count, dsig, dback, deps,
                           dwork, dstrain, strain_dt, fail_, gf, yo, geom, str, soft, wid, dg,
                           stream);
    e = cudaGetLastError();
    if (e != cudaSuccess) {
        (void)cudaStreamSynchronize(stream);
        return stage_cuda_error("material point kernel launch", e);
    }
    auto out = [&](double *dst, const double *src, size_t c) {
        if (e == cudaSuccess) e = get(dst, src, c, stream);
    };
    out(sig, dsig, 4 * n);
    out(back, dback, 4 * n);
    out(eps_p, deps, n);
    out(work, dwork, n);
    if (dgamma) out(dgamma, dg, n);
    if (dm) {
        out(damage->strength, str, n);
        out(damage->softening, soft, n);
        out(damage->width, wid, n);
    }
    const cudaError_t es = cudaStreamSynchronize(stream);
    if (e != cudaSuccess) return stage_cuda_error("copy out of the staging array failed", e);
    if (es != cudaSuccess) return stage_cuda_error("material point kernel", es);
    return NF_OK;
}
