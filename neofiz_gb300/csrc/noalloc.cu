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
// GPU that loads this library until the process exits. Its device address is looked up once
// per device (cudaGetSymbolAddress, with that device current) on the first call made on that
// device; make that first call before any stream capture. All calls share the array: a call
// overwrites every staging slot it reads before the kernel runs, so nothing stale is used, but
// two calls that overlap on the GPU (from two host threads, say) race on it.
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

nf_status stage_error(nf_status st, const char *msg) {
    set_thread_error(msg);
    return st;
}

// Device address of the staging array on the current device, looked up on first use.
nf_status stage_for_current_device(double **out) {
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= MAX_DEVICES)
        return stage_error(NF_EDEVICE, "no usable current CUDA device");
    std::lock_guard<std::mutex> guard(g_stage_lock);
    if (!g_stage_address[dev]) {
        void *p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_point_stage);
        if (e != cudaSuccess || !p) {
            char buf[256];
            snprintf(buf, sizeof buf, "cudaGetSymbolAddress of the staging array failed: %s",
                     cudaGetErrorString(e));
            return stage_error(NF_EDEVICE, buf);
        }
        g_stage_address[dev] = static_cast<double *>(p);
    }
    *out = g_stage_address[dev];
    return NF_OK;
}

bool put(double *dst, const double *src, size_t count) {
    return cudaMemcpy(dst, src, sizeof(double) * count, cudaMemcpyHostToDevice) == cudaSuccess;
}
bool get(double *dst, const double *src, size_t count) {
    return cudaMemcpy(dst, src, sizeof(double) * count, cudaMemcpyDeviceToHost) == cudaSuccess;
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
    nf_status st = stage_for_current_device(&base);
    if (st) return st;
    const size_t n = (size_t)count;
    const bool dm = damage && damage->failure_strain;
    double *dsig = base, *dback = dsig + 4 * n, *deps = dback + 4 * n, *dwork = deps + n;
    double *dstrain = dwork + n, *dg = dstrain + 4 * n;
    double *fail_ = nullptr, *gf = nullptr, *yo = nullptr, *geom = nullptr, *str = nullptr,
           *soft = nullptr, *wid = nullptr;
    bool ok = put(dsig, sig, 4 * n) && put(dback, back, 4 * n) && put(deps, eps_p, n) &&
              put(dwork, work, n) && put(dstrain, strain, 4 * n);
    if (dm) {
        fail_ = dg + n; gf = fail_ + n; yo = gf + n; geom = yo + n; str = geom + 5 * n;
        soft = str + n; wid = soft + n;
        ok = ok && put(fail_, damage->failure_strain, n) && put(gf, damage->fracture_energy, n) &&
             put(yo, damage->youngs_modulus, n) && put(geom, damage->geometry, 5 * n) &&
             put(str, damage->strength, n) && put(soft, damage->softening, n) &&
             put(wid, damage->width, n);
    }
    if (!ok) return stage_error(NF_EDEVICE, "copy into the staging array failed");
    launch_material_points(material_constants(*material, formulation), count, dsig, dback, deps,
                           dwork, dstrain, strain_dt, fail_, gf, yo, geom, str, soft, wid, dg, 0);
    cudaError_t e = cudaStreamSynchronize(0);
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e != cudaSuccess) {
        char buf[256];
        snprintf(buf, sizeof buf, "material point kernel: %s", cudaGetErrorString(e));
        return stage_error(NF_EDEVICE, buf);
    }
    ok = get(sig, dsig, 4 * n) && get(back, dback, 4 * n) && get(eps_p, deps, n) &&
         get(work, dwork, n);
    if (dgamma) ok = ok && get(dgamma, dg, n);
    if (dm) ok = ok && get(damage->strength, str, n) && get(damage->softening, soft, n) &&
                 get(damage->width, wid, n);
    if (!ok) return stage_error(NF_EDEVICE, "copy out of the staging array failed");
    return NF_OK;
}
