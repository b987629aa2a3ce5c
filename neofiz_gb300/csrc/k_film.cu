// k_film.cu -- Film.capture (src/main/java/org/neofiz/render/Film.java:148-224) on the device.
//
// The reference copies the whole state to the host for every frame and evaluates its field
// lambdas element by element. Here a capture is two kernels and two device-to-device copies
// enqueued on the solver's stream: the deformed node positions, the requested element fields
// and the live flags go into the film's next frame slot, the solver's scalars and the
// audit partial sums beside them; the host waits for nothing until it reads the frames back,
// once. The element fields follow the reference's accessors operation for operation in FP64
// and are kept in FP64, so a frame written out is the reference's frame digit for digit.
#include "nf_bodies.cuh"

#include <cstring>
#include <string>
#include <vector>

namespace nf {

constexpr int FILM_BLOCK = 256;
constexpr int FILM_MAX_FIELDS = 8;

struct FilmFields {
    int kind[FILM_MAX_FIELDS];
    int count;
};

__global__ void __launch_bounds__(FILM_BLOCK) k_film_nodes(Dev d, double *r, double *z) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.N) return;
    const double2 x = d.X0[i], u = d.U[i];
    r[i] = x.x + u.x;                            // Film.java:150-156
    z[i] = x.y + u.y;
}

// One element's field value, in the reference accessor's operation order.
__device__ double film_value(const Dev &d, int e, int kind) {
    const int ppe = d.ppe;
    switch (kind) {
        case NF_FILM_PLASTIC_STRAIN: {                   // ExplicitSolver.java:1897-1901
            double sum = 0.0;
            for (int g = 0; g < ppe; g++) sum += d.epsP[e * ppe + g];
            return sum / ppe;
        }
        case NF_FILM_DAMAGE: {                           // :1764-1772
            if (!d.hasDamage) return 0.0;
            double sum = 0.0;
            for (int g = 0; g < ppe; g++) {
                const int p = e * ppe + g;
                sum += damage_at(d.dStrength[p], d.dSoft[p], d.dFail[e], d.epsP[p]);
            }
            return sum / ppe;
        }
        case NF_FILM_VON_MISES_MPA:
        case NF_FILM_HOOP_STRESS_MPA: {                  // centroidStress, :1886-1894
            double s[4] = {0.0, 0.0, 0.0, 0.0};
            for (int g = 0; g < ppe; g++) {
                const double *q = d.sig + 4 * (size_t)(e * ppe + g);
                for (int c = 0; c < 4; c++) s[c] += q[c];
            }
            for (int c = 0; c < 4; c++) s[c] /= ppe;
            if (kind == NF_FILM_HOOP_STRESS_MPA) return s[2] / 1e6;
            // mises, Impact.java:229-232
            const double a = s[0] - s[1], b = s[1] - s[2], c = s[2] - s[0];
            return sqrt(0.5 * (a * a + b * b + c * c) + 3.0 * s[3] * s[3]) / 1e6;
        }
        case NF_FILM_SPEED: {                            // :895-902
            const int4 c = d.conn[e];
            const int nn[4] = {c.x, c.y, c.z, c.w};
            double sum = 0.0;
            for (int k = 0; k < 4; k++) {
                const double2 v = d.V[nn[k]];
                sum += sqrt(v.x * v.x + v.y * v.y);
            }
            return 0.25 * sum;
        }
    }
    return 0.0;
}

__global__ void __launch_bounds__(FILM_BLOCK) k_film_elements(Dev d, FilmFields f,
                                                             double *values, uint8_t *live) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= d.E) return;
    for (int k = 0; k < f.count; k++) values[(size_t)k * d.E + e] = film_value(d, e, f.kind[k]);
    live[e] = (d.gone != nullptr && d.gone[e]) ? 0 : 1;
}

}  // namespace nf

using namespace nf;

struct nf_film {
    Solver *S = nullptr;
    FilmFields fields{};
    int capacity = 0, frames = 0;
    size_t auditDoubles = 0;
    double *r = nullptr, *z = nullptr, *values = nullptr;
    uint8_t *live = nullptr;
    DevScalars *scal = nullptr;
    double *audit = nullptr;
    std::string err;
};

namespace {

nf_status film_fail(nf_film *f, nf_status st, const std::string &message) {
    f->err = message;
    return st;
}

void film_free(nf_film *f) {
    cudaFree(f->r); cudaFree(f->z); cudaFree(f->values); cudaFree(f->live);
    cudaFree(f->scal); cudaFree(f->audit);
}

// pressureAt (ExplicitSolver.java:1511-1520): the ramp's smoothstep of time
double pressure_at(const Dev &d, double t) {
    if (!(d.rampDuration > 0.0)) return d.targetPressure;
    const double s = t / d.rampDuration < 1.0 ? t / d.rampDuration : 1.0;
    return d.targetPressure * s * s * (3.0 - 2.0 * s);
}

thread_local std::string g_film_err;

}  // namespace

extern "C" {

const char *nf_film_last_error(const nf_film *f) {
    return f ? f->err.c_str() : g_film_err.c_str();
}

nf_status nf_film_create(nf_solver *h, const int32_t *fields, int32_t field_count,
                         int32_t capacity, nf_film **out) {
    *out = nullptr;
    Solver &S = *reinterpret_cast<Solver *>(h);
    if (field_count < 0 || field_count > FILM_MAX_FIELDS || (field_count > 0 && !fields)) {
        g_film_err = "a film takes 0 to 8 element fields";
        return NF_EINVAL;
    }
    if (capacity < 1) {
        g_film_err = "a film holds at least one frame";
        return NF_EINVAL;
    }
    for (int k = 0; k < field_count; k++)
        if (fields[k] < 0 || fields[k] >= NF_FILM_FIELD_KINDS) {
            g_film_err = "unknown film field " + std::to_string(fields[k]);
            return NF_EINVAL;
        }
    nf_film *f = new nf_film();
    f->S = &S;
    f->fields.count = field_count;
    for (int k = 0; k < field_count; k++) f->fields.kind[k] = fields[k];
    f->capacity = capacity;
    f->auditDoubles = audit_partial_doubles(S.d);
    const size_t N = S.N, E = S.E, C = capacity;
    cudaError_t e = cudaSuccess;
    auto A = [&](void **p, size_t bytes) {
        if (e == cudaSuccess) e = cudaMalloc(p, bytes ? bytes : 1);
    };
    A((void **)&f->r, 8 * N * C);
    A((void **)&f->z, 8 * N * C);
    A((void **)&f->values, 8 * E * C * (size_t)(field_count ? field_count : 1));
    A((void **)&f->live, E * C);
    A((void **)&f->scal, sizeof(DevScalars) * C);
    A((void **)&f->audit, sizeof(double) * f->auditDoubles * C);
    if (e != cudaSuccess) {
        g_film_err = std::string("film allocation failed: ") + cudaGetErrorString(e);
        film_free(f);
        delete f;
        return NF_ENOMEM;
    }
    *out = f;
    return NF_OK;
}

nf_status nf_film_destroy(nf_film *f) {
    if (!f) return NF_OK;
    if (f->S) cudaStreamSynchronize(f->S->stream);
    film_free(f);
    delete f;
    return NF_OK;
}

nf_status nf_film_capture(nf_film *f) {
    if (f->frames >= f->capacity)
        return film_fail(f, NF_ESTATE, "the film is full (" + std::to_string(f->capacity) +
                                           " frames)");
    Solver &S = *f->S;
    solver_state_to_double(S);                    // mixed precision: FP64 staging copy
    const size_t N = S.N, E = S.E, k = f->frames;
    Dev &d = S.d;
    if (N > 0)
        k_film_nodes<<<grid_for((long long)N, FILM_BLOCK), FILM_BLOCK, 0, S.stream>>>(
            d, f->r + k * N, f->z + k * N);
    if (E > 0)
        k_film_elements<<<grid_for((long long)E, FILM_BLOCK), FILM_BLOCK, 0, S.stream>>>(
            d, f->fields, f->values + k * E * (size_t)f->fields.count, f->live + k * E);
    cudaError_t e = cudaMemcpyAsync(f->scal + k, d.s, sizeof(DevScalars),
                                    cudaMemcpyDeviceToDevice, S.stream);
    if (e == cudaSuccess) {
        launch_audit_partials(S, f->audit + k * f->auditDoubles);
        e = cudaGetLastError();
    }
    if (e != cudaSuccess) return film_fail(f, NF_EDEVICE, cudaGetErrorString(e));
    S.launches += 4;
    f->frames++;
    return NF_OK;
}

nf_status nf_film_frames(nf_film *f, int32_t *count) {
    *count = f->frames;
    return NF_OK;
}

nf_status nf_film_clear(nf_film *f) {
    f->frames = 0;
    return NF_OK;
}

nf_status nf_film_read(nf_film *f, double *r, double *z, double *values, uint8_t *live,
                       nf_film_info *info, nf_audit *audits) {
    Solver &S = *f->S;
    const size_t N = S.N, E = S.E, C = f->frames;
    cudaError_t e = cudaSuccess;
    auto copy = [&](void *dst, const void *src, size_t bytes) {
        if (dst && bytes && e == cudaSuccess)
            e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, S.stream);
    };
    copy(r, f->r, 8 * N * C);
    copy(z, f->z, 8 * N * C);
    copy(values, f->values, 8 * E * C * (size_t)f->fields.count);
    copy(live, f->live, E * C);
    std::vector<DevScalars> sc(info ? C : 0);
    std::vector<double> partial(audits ? f->auditDoubles * C : 0);
    copy(sc.data(), f->scal, sizeof(DevScalars) * sc.size());
    copy(partial.data(), f->audit, sizeof(double) * partial.size());
    if (e != cudaSuccess) return film_fail(f, NF_EDEVICE, cudaGetErrorString(e));
    const nf_status st = solver_sync(S);
    if (st) return film_fail(f, st, nf_last_error(reinterpret_cast<nf_solver *>(&S)));
    for (size_t k = 0; k < C; k++) {
        if (info) {
            nf_film_info &o = info[k];
            o.time = sc[k].time;
            o.steps = sc[k].steps;
            o.eroded = sc[k].erodedCount;
            o.contact_pairs = sc[k].pairs;
            o.pressure = S.d.K > 0 ? pressure_at(S.d, sc[k].time) : 0.0;
        }
        if (audits) reduce_audit_partials(S, partial.data() + k * f->auditDoubles, &audits[k]);
    }
    return NF_OK;
}

}  // extern "C"
