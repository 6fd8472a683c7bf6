// Particle input and output between the caller's arrays and the packed
// per-atom records.
//
// tmps_atoms_assemble is AtomSystem.add_particles for a system's first
// particles (src/taichimps/atom.py:55-145): positions, radii, velocities and
// angular velocities in, the masses rmass = (4/3) pi r^3 density and moments
// of inertia 0.4 m r r formed here, tags 1..n unless given, forces zeroed.
// tmps_atoms_read is the per-atom fields' to_numpy() (the Taichi fields of
// atom.py:36-55 read back): one field, rows in insertion order.
//
// The caller's arrays may be device memory or page-locked host memory.  Host
// memory is read or written in place over the host link, by the same kernel
// that packs or unpacks the records: on this part SM loads and stores reach
// the link's rate (about 200 GB/s each way, the copy engines' rate too), so
// a staging copy through HBM would only add a pass and a launch.
#include "tmps_common.cuh"

using namespace tmps;

namespace {

constexpr int kBlock = 256;

// (4/3) pi in double, formed as the reference forms it: (4.0 / 3.0) * pi.
constexpr double kFourThirdsPi = (4.0 / 3.0) * 3.141592653589793;

// r^3 rounded once.  r*r is split exactly into p + e (the FMA residual), then
// p*r into h + l the same way; r^3 = h + l + e*r, and the small terms are
// summed before the one rounding of the total (the FMA form of Dekker's exact
// product: Ogita, Rump and Oishi, "Accurate sum and dot product", SIAM J. Sci.
// Comput. 26(6), 2005).  The result is the correctly rounded cube unless r^3
// lies within ~2^-106 (relative) of a rounding boundary, which is where a
// library pow(r, 3) -- the reference's numpy r**3 -- can also differ.
TMPS_DEV double cube_rn(double r) {
    const double p = __dmul_rn(r, r);
    const double e = __fma_rn(r, r, -p);
    const double h = __dmul_rn(p, r);
    const double l = __fma_rn(p, r, -h);
    return __dadd_rn(h, __fma_rn(e, r, l));
}

struct AssembleIn {
    const double* x;      // [n][3]
    const double* v;      // [n][3] or null (zero)
    const double* om;     // [n][3] or null (zero)
    const double* r;      // [n] or null (r_value for every atom)
    const double* dens;   // [n] or null (d_value for every atom)
    const int32_t* tag;   // [n] or null (1..n)
    double r_value, d_value;
};

__global__ void __launch_bounds__(kBlock) k_assemble(tmps_atoms a, AssembleIn in,
                                                     unsigned long long* __restrict__ rmax_bits) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int n = a.n;
    double r = 0.0;
    if (i < n) {
        const size_t k = 3 * (size_t)i;
        r = in.r ? in.r[i] : in.r_value;
        const double rho = in.dens ? in.dens[i] : in.d_value;
        const double x0 = in.x[k], x1 = in.x[k + 1], x2 = in.x[k + 2];
        double v0 = 0.0, v1 = 0.0, v2 = 0.0, w0 = 0.0, w1 = 0.0, w2 = 0.0;
        if (in.v) {
            v0 = in.v[k];
            v1 = in.v[k + 1];
            v2 = in.v[k + 2];
        }
        if (in.om) {
            w0 = in.om[k];
            w1 = in.om[k + 1];
            w2 = in.om[k + 2];
        }
        // atom.py:109-110 (vol = (4/3) pi r**3, rmass = vol density) and the
        // moment of inertia 0.4 m r r of nve_sphere.py:63, each product rounded
        // in order
        const double m = __dmul_rn(__dmul_rn(kFourThirdsPi, cube_rn(r)), rho);
        const double inertia = __dmul_rn(__dmul_rn(__dmul_rn(0.4, m), r), r);
        st4(a.xr, i, make_double4(x0, x1, x2, r));
        st4(a.vm, i, make_double4(v0, v1, v2, m));
        st4(a.om, i, make_double4(w0, w1, w2, inertia));
        a.tag[i] = in.tag ? in.tag[i] : i + 1;
        a.uid[i] = i;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            a.f[(size_t)c * n + i] = 0.0;
            a.torque[(size_t)c * n + i] = 0.0;
            a.x0[(size_t)c * n + i] = 0.0;
        }
        if (a.virial) {
#pragma unroll
            for (int c = 0; c < 6; ++c) a.virial[(size_t)c * n + i] = 0.0;
        }
    }
    // the largest radius: the bits of a non-negative double order as its value
    // (a negative radius counts as zero here; a NaN one wins, as in a max)
    unsigned long long b = r > 0.0 || r != r ? (unsigned long long)__double_as_longlong(r) : 0ull;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long t = __shfl_xor_sync(0xffffffffu, b, o);
        b = t > b ? t : b;
    }
    __shared__ unsigned long long wmax[kBlock / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) wmax[warp] = b;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long m = 0;
        for (int w = 0; w < kBlock / 32; ++w) m = wmax[w] > m ? wmax[w] : m;
        atomicMax(rmax_bits, m);
    }
}

__global__ void __launch_bounds__(kBlock) k_slot_of(const int32_t* __restrict__ uid, int n,
                                                    int32_t* __restrict__ slot_of) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        const int u = uid[i];
        if (u >= 0 && u < n) slot_of[u] = i;
    }
}

// Element q of the output is component c = q % w of the atom inserted as
// j = q / w: consecutive threads write consecutive words (whole lines over
// the host link) and read the records at their slots.
__global__ void __launch_bounds__(kBlock) k_read(tmps_atoms a, const int32_t* __restrict__ slot_of, int field,
                                                 int w, double* __restrict__ out) {
    const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int n = a.n;
    if (q >= (int64_t)n * w) return;
    const int j = (int)(q / w), c = (int)(q - (int64_t)j * w);
    const int s = slot_of[j];
    if (s < 0 || s >= n) {  // uid was not a permutation of 0..n-1
        out[q] = __longlong_as_double(0x7ff8000000000000ll);
        return;
    }
    double val;
    switch (field) {
        case TMPS_FIELD_X: val = a.xr[4 * (size_t)s + c]; break;
        case TMPS_FIELD_V: val = a.vm[4 * (size_t)s + c]; break;
        case TMPS_FIELD_OMEGA: val = a.om[4 * (size_t)s + c]; break;
        case TMPS_FIELD_RADIUS: val = a.xr[4 * (size_t)s + 3]; break;
        case TMPS_FIELD_RMASS: val = a.vm[4 * (size_t)s + 3]; break;
        case TMPS_FIELD_F: val = a.f[(size_t)c * n + s]; break;
        case TMPS_FIELD_TORQUE: val = a.torque[(size_t)c * n + s]; break;
        default: val = a.virial[(size_t)c * n + s]; break;
    }
    out[q] = val;
}

// Whether kernels can use the address p: device or managed memory, or
// page-locked host memory mapped for the device (then its device alias is
// returned).  Pageable host memory is refused.
bool device_view(const void* p, void** dev) {
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();  // a pointer the runtime does not know: clear the error it left
        return false;
    }
    if (at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged) {
        *dev = const_cast<void*>(p);
        return true;
    }
    if (at.type == cudaMemoryTypeHost && at.devicePointer != nullptr) {
        *dev = at.devicePointer;
        return true;
    }
    return false;
}

template <typename T>
bool view_opt(const T* p, const T** out) {
    if (!p) {
        *out = nullptr;
        return true;
    }
    void* d = nullptr;
    if (!device_view(p, &d)) return false;
    *out = static_cast<const T*>(d);
    return true;
}

int field_width(int field) {
    switch (field) {
        case TMPS_FIELD_X: case TMPS_FIELD_V: case TMPS_FIELD_OMEGA: case TMPS_FIELD_F: case TMPS_FIELD_TORQUE:
            return 3;
        case TMPS_FIELD_RADIUS: case TMPS_FIELD_RMASS:
            return 1;
        case TMPS_FIELD_VIRIAL:
            return 6;
        default:
            return 0;
    }
}

}  // namespace

extern "C" {

int tmps_atoms_assemble(const tmps_atoms* a, const double* x, const double* v, const double* omega,
                        const double* radius, double radius_value, const double* density, double density_value,
                        const int32_t* tag, double* d_max_radius, void* stream) {
    if (!a || a->n < 0 || !x || !d_max_radius || !a->xr || !a->vm || !a->om || !a->f || !a->torque || !a->tag ||
        !a->uid || !a->x0)
        return TMPS_ERR_BAD_ARG;
    AssembleIn in;
    void* dx = nullptr;
    if (!device_view(x, &dx)) return TMPS_ERR_BAD_ARG;
    in.x = static_cast<const double*>(dx);
    if (!view_opt(v, &in.v) || !view_opt(omega, &in.om) || !view_opt(radius, &in.r) ||
        !view_opt(density, &in.dens) || !view_opt(tag, &in.tag))
        return TMPS_ERR_BAD_ARG;
    in.r_value = radius_value;
    in.d_value = density_value;
    cudaStream_t s = (cudaStream_t)stream;
    if (cudaMemsetAsync(d_max_radius, 0, sizeof(double), s) != cudaSuccess) return TMPS_ERR_CUDA;
    if (a->n == 0) return TMPS_OK;
    k_assemble<<<grid_for(a->n, kBlock), kBlock, 0, s>>>(*a, in,
                                                          reinterpret_cast<unsigned long long*>(d_max_radius));
    note_launches(1);
    return cudaPeekAtLastError() == cudaSuccess ? TMPS_OK : TMPS_ERR_CUDA;
}

int tmps_atoms_read(const tmps_atoms* a, int32_t field, int32_t* d_slot_of, double* out, void* stream) {
    const int w = field_width(field);
    if (!a || a->n < 0 || w == 0 || !d_slot_of || !out || !a->uid) return TMPS_ERR_BAD_ARG;
    if (field == TMPS_FIELD_VIRIAL && !a->virial) return TMPS_ERR_BAD_ARG;
    if (a->n == 0) return TMPS_OK;
    void* dout = nullptr;
    if (!device_view(out, &dout)) return TMPS_ERR_BAD_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    k_slot_of<<<grid_for(a->n, kBlock), kBlock, 0, s>>>(a->uid, a->n, d_slot_of);
    k_read<<<grid_for((int64_t)a->n * w, kBlock), kBlock, 0, s>>>(*a, d_slot_of, field, w,
                                                                  static_cast<double*>(dout));
    note_launches(2);
    return cudaPeekAtLastError() == cudaSuccess ? TMPS_OK : TMPS_ERR_CUDA;
}

}  // extern "C"
