// State initialisation, distribution import/export, Courant number and
// steady-state residual kernels.
#include "device_common.cuh"
#include "kernels.h"

namespace dugks {
namespace {

int grid_for(long long n, int threads, int sms) {
    long long b = (n + threads - 1) / threads;
    long long cap = (long long)sms * 32;
    return (int)(b < cap ? (b > 0 ? b : 1) : cap);
}

// discreteVelocity::initDFtoEq (discreteVelocity.C:220-249): Shakhov with q = 0.
template <typename S>
__global__ void k_init_state(StepArgs a, S* gT, S* hT, double gscale) {
    const long long n = (long long)a.nC * a.Vp;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        int c = (int)(i / a.Vp), v = (int)(i - (long long)c * a.Vp);
        if (v >= a.nV) {
            gT[i] = S(0);
            if (a.hasH) hT[i] = S(0);
            continue;
        }
        double ge, he;
        shakhov_ref(a.rho[c], a.U[3 * c], a.U[3 * c + 1], a.U[3 * c + 2], a.T[c], 0.0, 0.0, 0.0, a.xi[v],
                    a.xi[a.Vp + v], a.xi[2 * a.Vp + v], a.R, a.Pr, a.D, a.K, ge, he);
        gT[i] = S(ge * gscale);
        if (a.hasH) hT[i] = S(he * gscale);
        if (v == 0) a.tau[c] = tau_ref(a.T[c], a.rho[c], a.muRef, a.omega, a.Tref, a.R);
    }
}

template <typename S>
__global__ void k_export(StepArgs a, const S* src, double* dst, double inv) {
    const long long n = (long long)a.nC * a.nV;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        int c = (int)(i / a.nV), v = (int)(i - (long long)c * a.nV);
        dst[i] = (double)src[(long long)c * a.Vp + v] * inv;
    }
}

template <typename S>
__global__ void k_import(StepArgs a, const double* src, S* dst, double scale) {
    const long long n = (long long)a.nC * a.nV;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        int c = (int)(i / a.nV), v = (int)(i - (long long)c * a.nV);
        dst[(long long)c * a.Vp + v] = S(src[i] * scale);
    }
}

// Deterministic two-stage reductions over all SMs: kRedBlocks fixed blocks
// write partials, one block adds them in a fixed order.
constexpr int kRedBlocks = 128, kRedThreads = 256;

template <int N>
__global__ void k_reduce_partials(const double* part, int nmax, double* out) {
    __shared__ double red[32 * N];
    double s[N];
    double mx = 0.0;
    for (int i = 0; i < N; ++i) s[i] = threadIdx.x < kRedBlocks ? part[threadIdx.x * (N + 1) + i] : 0.0;
    if (threadIdx.x < kRedBlocks && nmax) mx = part[threadIdx.x * (N + 1) + N];
    block_sum<N>(s, red);
    for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    __shared__ double redm[32];
    if ((threadIdx.x & 31) == 0) redm[threadIdx.x >> 5] = mx;
    __syncthreads();
    if (threadIdx.x == 0) {
        double m = 0.0;
        for (int i = 0; i < (int)(blockDim.x >> 5); ++i) m = fmax(m, redm[i]);
        if (nmax) out[0] = m;
        for (int i = 0; i < N; ++i) out[nmax + i] = s[i];
    }
}

// fvDVM::getCoNum (fvDVM.C:1111-1119): per internal face deltaCoeff * (|U_f| + sqrt(D) xi_max);
// partial {sum, max} per block.
__global__ void k_conum(StepArgs a, const double* dcI, double xi_max, double* part) {
    __shared__ double red[32];
    __shared__ double redm[32];
    double s[1] = {0.0};
    double mx = 0.0;
    const double sq = sqrt((double)a.D) * xi_max;
    for (int f = blockIdx.x * blockDim.x + threadIdx.x; f < a.nI; f += gridDim.x * blockDim.x) {
        double ux = a.UF[3 * f], uy = a.UF[3 * f + 1], uz = a.UF[3 * f + 2];
        double u = dcI[f] * (sqrt(ux * ux + uy * uy + uz * uz) + sq);
        s[0] += u;
        mx = fmax(mx, u);
    }
    block_sum<1>(s, red);
    for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if ((threadIdx.x & 31) == 0) redm[threadIdx.x >> 5] = mx;
    __syncthreads();
    if (threadIdx.x == 0) {
        double m = 0.0;
        for (int i = 0; i < (int)(blockDim.x >> 5); ++i) m = fmax(m, redm[i]);
        part[blockIdx.x * 2] = s[0];
        part[blockIdx.x * 2 + 1] = m;
    }
}

// dugksFoam.C:88-107 residuals; then the "old" fields take the current ones.
// Partial sums per block.
__global__ void k_residual(StepArgs a, double* Uo, double* To, double* ro, double* part) {
    __shared__ double red[32 * 6];
    double s[6] = {0, 0, 0, 0, 0, 0};
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < a.nC; c += gridDim.x * blockDim.x) {
        double dx = a.U[3 * c] - Uo[3 * c], dy = a.U[3 * c + 1] - Uo[3 * c + 1], dz = a.U[3 * c + 2] - Uo[3 * c + 2];
        s[0] += sqrt(dx * dx + dy * dy + dz * dz);
        s[1] += sqrt(a.U[3 * c] * a.U[3 * c] + a.U[3 * c + 1] * a.U[3 * c + 1] + a.U[3 * c + 2] * a.U[3 * c + 2]);
        s[2] += fabs(a.T[c] - To[c]);
        s[3] += a.T[c];
        s[4] += fabs(a.rho[c] - ro[c]);
        s[5] += a.rho[c];
        Uo[3 * c] = a.U[3 * c]; Uo[3 * c + 1] = a.U[3 * c + 1]; Uo[3 * c + 2] = a.U[3 * c + 2];
        To[c] = a.T[c];
        ro[c] = a.rho[c];
    }
    block_sum<6>(s, red);
    if (threadIdx.x == 0)
        for (int i = 0; i < 6; ++i) part[blockIdx.x * 7 + i] = s[i];
}

}  // namespace

template <typename S>
void launch_init_state(const StepArgs& a, S* gT, S* hT, double gscale, int sms, cudaStream_t s) {
    k_init_state<S><<<grid_for((long long)a.nC * a.Vp, 256, sms), 256, 0, s>>>(a, gT, hT, gscale);
}
template <typename S>
void launch_export_dist(const StepArgs& a, const S* src, double* dst, double inv, int sms, cudaStream_t s) {
    k_export<S><<<grid_for((long long)a.nC * a.nV, 256, sms), 256, 0, s>>>(a, src, dst, inv);
}
template <typename S>
void launch_import_dist(const StepArgs& a, const double* src, S* dst, double scale, int sms, cudaStream_t s) {
    k_import<S><<<grid_for((long long)a.nC * a.nV, 256, sms), 256, 0, s>>>(a, src, dst, scale);
}
// out: {max, sum}; scratch: kRedBlocks * 2 doubles past out + 8
void launch_conum(const StepArgs& a, const double* dcI, double xi_max, double* out, cudaStream_t s) {
    double* part = out + 8;
    k_conum<<<kRedBlocks, kRedThreads, 0, s>>>(a, dcI, xi_max, part);
    k_reduce_partials<1><<<1, kRedBlocks, 0, s>>>(part, 1, out);
}
// out: 6 sums; scratch: kRedBlocks * 7 doubles past out + 8
void launch_residual(const StepArgs& a, double* Uo, double* To, double* ro, double* out, cudaStream_t s) {
    double* part = out + 8;
    k_residual<<<kRedBlocks, kRedThreads, 0, s>>>(a, Uo, To, ro, part);
    k_reduce_partials<6><<<1, kRedBlocks, 0, s>>>(part, 0, out);
}

template void launch_init_state<double>(const StepArgs&, double*, double*, double, int, cudaStream_t);
template void launch_init_state<float>(const StepArgs&, float*, float*, double, int, cudaStream_t);
template void launch_export_dist<double>(const StepArgs&, const double*, double*, double, int, cudaStream_t);
template void launch_export_dist<float>(const StepArgs&, const float*, double*, double, int, cudaStream_t);
template void launch_import_dist<double>(const StepArgs&, const double*, double*, double, int, cudaStream_t);
template void launch_import_dist<float>(const StepArgs&, const double*, float*, double, int, cudaStream_t);

}  // namespace dugks

// 1 when this library was compiled with the device-side index checks.
extern "C" int dugks_checked_build(void) {
#if defined(DUGKS_CHECKED) && DUGKS_CHECKED
    return 1;
#else
    return 0;
#endif
}
