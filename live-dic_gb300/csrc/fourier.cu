// Global-translation initializer by linear phase correlation on the GPU
// (reference: fourier.py:16-111, FourierInitializer, which runs it in NumPy
// float64 on the CPU).
//
// Reference side, once: the chosen size x size window (size = a power of two
// <= 1024) minus its mean over ROI-allowed pixels, zeroed outside the ROI,
// 2x2-averaged to half x half samples, Hann-tapered, zero-padded back to
// size x size and transformed.  Per target: the same window (mean over all
// pixels), the same reduction and taper, forward FFT, normalised cross power
// spectrum F_cur conj(F_ref) / max(|.|, 1e-12), inverse FFT, the peak
// (first maximum in row-major order), its score against the background
// outside the wrapped 11 x 11 neighbourhood, the even-pixel shift, the
// window overlap, and the normalised correlation of the reduced samples over
// the overlapping, ROI-allowed region.  out = {dx, dy, peak score, overlap,
// correlation, peak, target window standard deviation}.
//
// Transforms are radix-2 decimation-in-time in float64 (the reference's
// precision): one CTA per row or column line, the line in shared memory in
// bit-reversed order, twiddles from sincospi.  Sums are exact integers where
// the inputs are bytes and float64 elsewhere.
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "engine.h"

using gbdic::check_cuda;
using gbdic::fail;
using gbdic::Failure;

namespace {

__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
    return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// Integer sum, count and sum of squares of the window bytes (allowed pixels).
__global__ void window_sum_kernel(const uint8_t *img, long long pitch, int x0, int y0, int size, const uint8_t *allowed,
                                  unsigned long long *sums) {
    unsigned long long s = 0, n = 0, q = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < size * size; i += gridDim.x * blockDim.x) {
        const int r = i / size, c = i % size;
        if (allowed && !allowed[i]) continue;
        const unsigned long long v = img[(size_t)(y0 + r) * pitch + x0 + c];
        s += v;
        q += v * v;
        ++n;
    }
    for (int off = 16; off > 0; off >>= 1) {
        s += __shfl_down_sync(0xffffffffu, s, off);
        n += __shfl_down_sync(0xffffffffu, n, off);
        q += __shfl_down_sync(0xffffffffu, q, off);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(&sums[0], s);
        atomicAdd(&sums[1], n);
        atomicAdd(&sums[2], q);
    }
}

// Reduced samples (2x2 means of the mean-free, ROI-zeroed window), their
// taper into the zero-padded transform input, and the allowed samples.
__global__ void reduce_taper_kernel(const uint8_t *img, long long pitch, int x0, int y0, int size,
                                    const uint8_t *allowed, const unsigned long long *sums, const double *taper,
                                    double *samples, uint8_t *allowed_samples, double2 *spectrum_in) {
    const int half = size / 2;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= size * size) return;
    const int r = i / size, c = i % size;
    if (r >= half || c >= half) {
        spectrum_in[i] = make_double2(0.0, 0.0);
        return;
    }
    const double mean = (double)sums[0] / (double)sums[1];
    double acc = 0.0;
    bool all = true;
    for (int dy = 0; dy < 2; ++dy)
        for (int dx = 0; dx < 2; ++dx) {
            const int rr = 2 * r + dy, cc = 2 * c + dx;
            const bool ok = allowed == nullptr || allowed[rr * size + cc];
            all = all && ok;
            const double v = ((double)img[(size_t)(y0 + rr) * pitch + x0 + cc] - mean) * (ok ? 1.0 : 0.0);
            acc += v;
        }
    const double reduced = acc / 4.0;
    samples[r * half + c] = reduced;
    if (allowed_samples) allowed_samples[r * half + c] = all ? 1 : 0;
    spectrum_in[i] = make_double2(reduced * taper[r] * taper[c], 0.0);
}

// Twiddle factors of an n-point transform, k < n/2: (cos, sin) of
// sign * 2 pi k / n for sign -1 (forward, first half) and +1 (inverse).
// Stage s of the transform uses entry pos * (n / 2^s), whose argument
// sign * 2 * pos / 2^s is the same double, so the factors equal a per-stage
// sincospi() bit for bit.
__global__ void twiddle_kernel(double2 *tw, int n) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n / 2) return;
    double sn, cs;
    sincospi(-1.0 * 2.0 * (double)k / (double)n, &sn, &cs);
    tw[k] = make_double2(cs, sn);
    sincospi(1.0 * 2.0 * (double)k / (double)n, &sn, &cs);
    tw[n / 2 + k] = make_double2(cs, sn);
}

// In-place radix-2 transform of `lines` lines of n points: element k of line
// l at data[l * dist + k * step]; twiddles from `tw` (the forward or inverse
// half of the table), unscaled.
__global__ void fft_lines_kernel(double2 *data, int n, int logn, long long step, long long dist, const double2 *tw) {
    extern __shared__ double2 line[];
    double2 *base = data + (size_t)blockIdx.x * dist;
    for (int k = threadIdx.x; k < n; k += blockDim.x) line[__brev((unsigned)k) >> (32 - logn)] = base[(size_t)k * step];
    __syncthreads();
    for (int s = 1; s <= logn; ++s) {
        const int m = 1 << s, h = m >> 1;
        for (int j = threadIdx.x; j < n / 2; j += blockDim.x) {
            const int pos = j & (h - 1), i0 = (j >> (s - 1)) * m + pos, i1 = i0 + h;
            const double2 t = cmul(__ldg(tw + (pos << (logn - s))), line[i1]), u = line[i0];
            line[i0] = make_double2(u.x + t.x, u.y + t.y);
            line[i1] = make_double2(u.x - t.x, u.y - t.y);
        }
        __syncthreads();
    }
    for (int k = threadIdx.x; k < n; k += blockDim.x) base[(size_t)k * step] = line[k];
}

__global__ void cross_power_kernel(double2 *cur, const double2 *ref, int count) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    const double2 a = cur[i], b = ref[i];
    const double2 c = make_double2(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);  // a conj(b)
    const double m = fmax(sqrt(c.x * c.x + c.y * c.y), 1e-12);
    cur[i] = make_double2(c.x / m, c.y / m);
}

// Stage 1 of the peak search over the correlation (real part / n^2): per CTA
// the first maximum (lowest index on ties) and the sums of the values and
// of their squares.
constexpr int kPeakCtas = 128, kPeakThreads = 256;

__global__ void __launch_bounds__(kPeakThreads) peak_partial_kernel(const double2 *corr, int size, double *pbest,
                                                                     int *pidx, double *psum, double *psq) {
    const int n = size * size;
    const double scale = 1.0 / (double)n;
    double best = -1e300, s = 0.0, q = 0.0;
    int best_i = 0x7fffffff;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const double v = corr[i].x * scale;
        s += v;
        q += v * v;
        if (v > best) { best = v; best_i = i; }
    }
    __shared__ double sb[kPeakThreads], ss[kPeakThreads], sq[kPeakThreads];
    __shared__ int si[kPeakThreads];
    sb[threadIdx.x] = best; si[threadIdx.x] = best_i; ss[threadIdx.x] = s; sq[threadIdx.x] = q;
    __syncthreads();
    for (int off = blockDim.x / 2; off > 0; off >>= 1) {
        if (threadIdx.x < off) {
            const double b2 = sb[threadIdx.x + off];
            const int i2 = si[threadIdx.x + off];
            if (b2 > sb[threadIdx.x] || (b2 == sb[threadIdx.x] && i2 < si[threadIdx.x])) {
                sb[threadIdx.x] = b2;
                si[threadIdx.x] = i2;
            }
            ss[threadIdx.x] += ss[threadIdx.x + off];
            sq[threadIdx.x] += sq[threadIdx.x + off];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        pbest[blockIdx.x] = sb[0];
        pidx[blockIdx.x] = si[0];
        psum[blockIdx.x] = ss[0];
        psq[blockIdx.x] = sq[0];
    }
}

// Stage 2 (one CTA): combine the partials in a fixed order, then the mean
// and deviation of the correlation outside the wrapped 11 x 11 block
// around the peak.
__global__ void __launch_bounds__(kPeakCtas) peak_final_kernel(const double2 *corr, int size, const double *pbest,
                                                                const int *pidx, const double *psum,
                                                                const double *psq, double *out) {
    __shared__ double sb[kPeakCtas], ss[kPeakCtas], sq[kPeakCtas];
    __shared__ int si[kPeakCtas];
    sb[threadIdx.x] = pbest[threadIdx.x]; si[threadIdx.x] = pidx[threadIdx.x];
    ss[threadIdx.x] = psum[threadIdx.x]; sq[threadIdx.x] = psq[threadIdx.x];
    __syncthreads();
    for (int off = blockDim.x / 2; off > 0; off >>= 1) {
        if (threadIdx.x < off) {
            const double b2 = sb[threadIdx.x + off];
            const int i2 = si[threadIdx.x + off];
            if (b2 > sb[threadIdx.x] || (b2 == sb[threadIdx.x] && i2 < si[threadIdx.x])) {
                sb[threadIdx.x] = b2;
                si[threadIdx.x] = i2;
            }
            ss[threadIdx.x] += ss[threadIdx.x + off];
            sq[threadIdx.x] += sq[threadIdx.x + off];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        const int n = size * size;
        const double scale = 1.0 / (double)n;
        const int py = si[0] / size, px = si[0] % size;
        double bs = 0.0, bq = 0.0;
        for (int dy = -5; dy <= 5; ++dy)
            for (int dx = -5; dx <= 5; ++dx) {
                const int r = ((py + dy) % size + size) % size, c = ((px + dx) % size + size) % size;
                const double v = corr[r * size + c].x * scale;
                bs += v;
                bq += v * v;
            }
        const double m = (double)(n - 121);
        const double mean = (ss[0] - bs) / m;
        const double var = fmax((sq[0] - bq) / m - mean * mean, 0.0);
        out[0] = sb[0];
        out[1] = (double)px;
        out[2] = (double)py;
        out[3] = mean;
        out[4] = sqrt(var);
    }
}

// Normalised correlation of reference and current reduced samples over the
// overlap for shift (sx, sy) in samples, allowed reference samples only:
// per-CTA partial sums (stage 1), combined in a fixed order (stage 2).
constexpr int kCorrCtas = 64, kCorrThreads = 256;

__global__ void __launch_bounds__(kCorrThreads) overlap_partial_kernel(const double *ref, const uint8_t *allowed,
                                                                        const double *cur, int half, int sx, int sy,
                                                                        double *partial) {
    const int y0 = max(0, -sy), y1 = min(half, half - sy), x0 = max(0, -sx), x1 = min(half, half - sx);
    const int w = max(0, x1 - x0), h = max(0, y1 - y0);
    double sa = 0, sb = 0, sab = 0, saa = 0, sbb = 0, n = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < w * h; i += gridDim.x * blockDim.x) {
        const int r = y0 + i / w, c = x0 + i % w;
        if (!allowed[r * half + c]) continue;
        const double a = ref[r * half + c], b = cur[(r + sy) * half + (c + sx)];
        sa += a; sb += b; sab += a * b; saa += a * a; sbb += b * b; n += 1.0;
    }
    __shared__ double red[6][kCorrThreads];
    const double v[6] = {sa, sb, sab, saa, sbb, n};
    for (int k = 0; k < 6; ++k) red[k][threadIdx.x] = v[k];
    __syncthreads();
    for (int off = blockDim.x / 2; off > 0; off >>= 1) {
        if (threadIdx.x < off)
            for (int k = 0; k < 6; ++k) red[k][threadIdx.x] += red[k][threadIdx.x + off];
        __syncthreads();
    }
    if (threadIdx.x < 6) partial[threadIdx.x * kCorrCtas + blockIdx.x] = red[threadIdx.x][0];
}

__global__ void __launch_bounds__(kCorrCtas) overlap_final_kernel(const double *partial, double *out) {
    __shared__ double red[6][kCorrCtas];
    for (int k = 0; k < 6; ++k) red[k][threadIdx.x] = partial[k * kCorrCtas + threadIdx.x];
    __syncthreads();
    for (int off = blockDim.x / 2; off > 0; off >>= 1) {
        if (threadIdx.x < off)
            for (int k = 0; k < 6; ++k) red[k][threadIdx.x] += red[k][threadIdx.x + off];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        const double cnt = red[5][0];
        double corr = 0.0;
        if (cnt > 0) {
            const double ma = red[0][0] / cnt, mb = red[1][0] / cnt;
            const double cab = red[2][0] - cnt * ma * mb;
            const double caa = fmax(red[3][0] - cnt * ma * ma, 0.0), cbb = fmax(red[4][0] - cnt * mb * mb, 0.0);
            const double norm = sqrt(caa) * sqrt(cbb);
            corr = norm > 0 ? cab / norm : 0.0;
        }
        out[5] = corr;
    }
}

// Accepted shift of the last phase correlation written into rows of affine
// parameters without a host round trip: the integer peak shift (the same
// unwrapping as the host path), accepted when the target window has texture
// (standard deviation >= 1), the peak score reaches 8 and the overlap 0.25;
// rows[i * pitch] = dx * multiplier, rows[i * pitch + 3] = dy * multiplier,
// zero when rejected.  The sample-correlation test of the host path needs the
// shift on the host to launch and is not applied here.
__global__ void shift_rows_kernel(const double *result, const unsigned long long *sums, int size, float multiplier,
                                  float *rows, int count, int pitch) {
    __shared__ float su, sv;
    if (threadIdx.x == 0) {
        const double wn = (double)sums[1], wmean = wn > 0 ? (double)sums[0] / wn : 0.0;
        const double texture = wn > 0 ? sqrt(fmax((double)sums[2] / wn - wmean * wmean, 0.0)) : 0.0;
        const int half = size / 2, px = (int)result[1], py = (int)result[2];
        const int dx = 2 * (px < half ? px : px - size), dy = 2 * (py < half ? py : py - size);
        const double sd = result[4];
        const double score = (result[0] - result[3]) / (sd > 1e-12 ? sd : 1e-12);
        const double ox = (double)max(size - abs(dx), 0), oy = (double)max(size - abs(dy), 0);
        const double overlap = ox * oy / ((double)size * size);
        const bool ok = texture >= 1.0 && score >= 8.0 && overlap >= 0.25;
        su = ok ? (float)dx * multiplier : 0.0f;
        sv = ok ? (float)dy * multiplier : 0.0f;
    }
    __syncthreads();
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
        rows[(size_t)i * pitch] = su;
        rows[(size_t)i * pitch + 3] = sv;
    }
}

int log2i(int n) {
    int l = 0;
    while ((1 << l) < n) ++l;
    return l;
}

thread_local std::string g_fourier_error;

}  // namespace

struct gbdic_fourier {
    int device = 0, size = 0, half = 0, logn = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t fork = nullptr, join = nullptr;
    gbdic::DeviceBuffer window, allowed, taper, ref_spectrum, ref_samples, allowed_samples, cur_samples, work, sums,
        result, twiddle, partials;
    gbdic::HostBuffer host_window, host_result;
    std::string error;
    ~gbdic_fourier() {
        cudaSetDevice(device);
        if (stream) {
            cudaStreamSynchronize(stream);
            cudaStreamDestroy(stream);
        }
        if (fork) cudaEventDestroy(fork);
        if (join) cudaEventDestroy(join);
    }
    void transform(double sign) { transform(sign, stream); }
    void transform(double sign, cudaStream_t st) {
        const int n = size;
        const size_t smem = (size_t)n * sizeof(double2);
        const int threads = n / 2 < 512 ? n / 2 : 512;
        double2 *d = work.as<double2>();
        const double2 *tw = twiddle.as<double2>() + (sign < 0.0 ? 0 : n / 2);
        fft_lines_kernel<<<n, threads, smem, st>>>(d, n, logn, 1, n, tw);  // rows
        check_cuda(cudaGetLastError(), "FFT rows");
        fft_lines_kernel<<<n, threads, smem, st>>>(d, n, logn, n, 1, tw);  // columns
        check_cuda(cudaGetLastError(), "FFT columns");
    }
    // window bytes (device, dense size x size) -> work (spectrum), samples
    void spectrum_of(const uint8_t *win, const uint8_t *allow, double *samples, uint8_t *allowed_out) {
        spectrum_of(win, allow, samples, allowed_out, stream);
    }
    void spectrum_of(const uint8_t *win, const uint8_t *allow, double *samples, uint8_t *allowed_out,
                     cudaStream_t st) {
        check_cuda(cudaMemsetAsync(sums.get(), 0, 3 * sizeof(unsigned long long), st), "clear");
        window_sum_kernel<<<256, 256, 0, st>>>(win, size, 0, 0, size, allow, sums.as<unsigned long long>());
        check_cuda(cudaGetLastError(), "window mean");
        const int count = size * size;
        reduce_taper_kernel<<<(count + 255) / 256, 256, 0, st>>>(win, size, 0, 0, size, allow,
                                                                  sums.as<unsigned long long>(), taper.as<double>(),
                                                                  samples, allowed_out, work.as<double2>());
        check_cuda(cudaGetLastError(), "reduction and taper");
        transform(-1.0, st);
    }
};

namespace {

template <typename F>
int fguarded(gbdic_fourier *f, F &&fn) {
    if (!f) {
        g_fourier_error = "null handle";
        return GBDIC_EINVAL;
    }
    try {
        check_cuda(cudaSetDevice(f->device), "cudaSetDevice");
        fn();
        return GBDIC_OK;
    } catch (const Failure &x) {
        f->error = x.message;
        return x.code;
    } catch (const std::exception &x) {
        f->error = x.what();
        return GBDIC_ECUDA;
    }
}

}  // namespace

extern "C" {

const char *gbdic_fourier_last_error(const gbdic_fourier *f) { return f ? f->error.c_str() : g_fourier_error.c_str(); }

int gbdic_fourier_create(int32_t device, const uint8_t *window, const uint8_t *allowed, int32_t size,
                         gbdic_fourier **out) {
    if (!out || !window) {
        g_fourier_error = "window and output handle are required";
        return GBDIC_EINVAL;
    }
    *out = nullptr;
    if (size < 32 || size > 1024 || (size & (size - 1))) {
        g_fourier_error = "window size must be a power of two from 32 to 1024";
        return GBDIC_EINVAL;
    }
    auto *f = new gbdic_fourier();
    try {
        f->device = device;
        check_cuda(cudaSetDevice(device), "cudaSetDevice");
        check_cuda(cudaStreamCreateWithFlags(&f->stream, cudaStreamNonBlocking), "stream");
        check_cuda(cudaEventCreateWithFlags(&f->fork, cudaEventDisableTiming), "event");
        check_cuda(cudaEventCreateWithFlags(&f->join, cudaEventDisableTiming), "event");
        f->size = size;
        f->half = size / 2;
        f->logn = log2i(size);
        const size_t px = (size_t)size * size, hpx = (size_t)f->half * f->half;
        f->window.ensure(px);
        f->taper.ensure((size_t)f->half * sizeof(double));
        f->ref_spectrum.ensure(px * sizeof(double2));
        f->work.ensure(px * sizeof(double2));
        f->ref_samples.ensure(hpx * sizeof(double));
        f->cur_samples.ensure(hpx * sizeof(double));
        f->allowed_samples.ensure(hpx);
        f->sums.ensure(3 * sizeof(unsigned long long));
        f->result.ensure(8 * sizeof(double));
        f->twiddle.ensure((size_t)size * sizeof(double2));
        f->partials.ensure((size_t)(4 * kPeakCtas + 6 * kCorrCtas) * sizeof(double));
        f->host_window.ensure(px);
        f->host_result.ensure(8 * sizeof(double));
        twiddle_kernel<<<(size / 2 + 255) / 256, 256, 0, f->stream>>>(f->twiddle.as<double2>(), size);
        check_cuda(cudaGetLastError(), "twiddles");
        // Hann taper of `half` points: 0.5 - 0.5 cos(2 pi k / (half - 1)).
        std::vector<double> taper((size_t)f->half);
        const double pi = 3.14159265358979323846;
        for (int k = 0; k < f->half; ++k) taper[(size_t)k] = 0.5 - 0.5 * cos(2.0 * pi * k / (double)(f->half - 1));
        check_cuda(cudaMemcpy(f->taper.get(), taper.data(), taper.size() * sizeof(double), cudaMemcpyHostToDevice), "taper");
        check_cuda(cudaMemcpy(f->window.get(), window, px, cudaMemcpyHostToDevice), "window");
        const uint8_t *allow = nullptr;
        if (allowed) {
            f->allowed.ensure(px);
            check_cuda(cudaMemcpy(f->allowed.get(), allowed, px, cudaMemcpyHostToDevice), "ROI window");
            allow = f->allowed.as<uint8_t>();
        }
        f->spectrum_of(f->window.as<uint8_t>(), allow, f->ref_samples.as<double>(), f->allowed_samples.as<uint8_t>());
        check_cuda(cudaMemcpyAsync(f->ref_spectrum.get(), f->work.get(), px * sizeof(double2), cudaMemcpyDeviceToDevice,
                                   f->stream), "spectrum copy");
        check_cuda(cudaStreamSynchronize(f->stream), "reference spectrum");
    } catch (const Failure &x) {
        g_fourier_error = x.message;
        delete f;
        return x.code;
    }
    *out = f;
    return GBDIC_OK;
}

int gbdic_fourier_destroy(gbdic_fourier *f) {
    delete f;
    return GBDIC_OK;
}

int gbdic_fourier_estimate(gbdic_fourier *f, const uint8_t *frame, int64_t row_stride, int32_t height, int32_t x,
                           int32_t y, int32_t device_frame, double *out) {
    return fguarded(f, [&] {
        if (!frame || !out) fail(GBDIC_EINVAL, "frame and output are required");
        const int n = f->size;
        if (row_stride < x + n || x < 0 || y < 0 || y + n > height) fail(GBDIC_EINVAL, "window outside the frame");
        if (device_frame) {
            check_cuda(cudaMemcpy2DAsync(f->window.get(), n, frame + (size_t)y * row_stride + x, (size_t)row_stride, n, n,
                                         cudaMemcpyDeviceToDevice, f->stream), "window copy");
        } else {
            uint8_t *dst = f->host_window.as<uint8_t>();
            for (int r = 0; r < n; ++r) std::memcpy(dst + (size_t)r * n, frame + (size_t)(y + r) * row_stride + x, n);
            check_cuda(cudaMemcpyAsync(f->window.get(), dst, (size_t)n * n, cudaMemcpyHostToDevice, f->stream),
                       "window upload");
        }
        f->spectrum_of(f->window.as<uint8_t>(), nullptr, f->cur_samples.as<double>(), nullptr);
        const int count = n * n;
        cross_power_kernel<<<(count + 255) / 256, 256, 0, f->stream>>>(f->work.as<double2>(), f->ref_spectrum.as<double2>(),
                                                                      count);
        check_cuda(cudaGetLastError(), "cross power");
        f->transform(+1.0);
        double *pb = f->partials.as<double>();
        peak_partial_kernel<<<kPeakCtas, kPeakThreads, 0, f->stream>>>(
            f->work.as<double2>(), n, pb, reinterpret_cast<int *>(pb + kPeakCtas), pb + 2 * kPeakCtas,
            pb + 3 * kPeakCtas);
        check_cuda(cudaGetLastError(), "peak");
        peak_final_kernel<<<1, kPeakCtas, 0, f->stream>>>(f->work.as<double2>(), n, pb,
                                                          reinterpret_cast<const int *>(pb + kPeakCtas),
                                                          pb + 2 * kPeakCtas, pb + 3 * kPeakCtas,
                                                          f->result.as<double>());
        check_cuda(cudaGetLastError(), "peak");
        check_cuda(cudaMemcpyAsync(f->host_result.as<double>(), f->result.get(), 5 * sizeof(double), cudaMemcpyDeviceToHost,
                                   f->stream), "peak readback");
        unsigned long long window_sums[3];
        check_cuda(cudaMemcpyAsync(window_sums, f->sums.get(), sizeof(window_sums), cudaMemcpyDeviceToHost, f->stream),
                   "window statistics");
        check_cuda(cudaStreamSynchronize(f->stream), "phase correlation");
        double *r = f->host_result.as<double>();
        const double wn = (double)window_sums[1], wmean = (double)window_sums[0] / wn;
        out[6] = sqrt(fmax((double)window_sums[2] / wn - wmean * wmean, 0.0));
        const int half = f->half;
        const int px = (int)r[1], py = (int)r[2];
        const int dx = 2 * (px < half ? px : px - n), dy = 2 * (py < half ? py : py - n);
        double *pc = f->partials.as<double>() + 4 * kPeakCtas;
        overlap_partial_kernel<<<kCorrCtas, kCorrThreads, 0, f->stream>>>(
            f->ref_samples.as<double>(), f->allowed_samples.as<uint8_t>(), f->cur_samples.as<double>(), half, dx / 2,
            dy / 2, pc);
        check_cuda(cudaGetLastError(), "overlap correlation");
        overlap_final_kernel<<<1, kCorrCtas, 0, f->stream>>>(pc, f->result.as<double>());
        check_cuda(cudaGetLastError(), "overlap correlation");
        check_cuda(cudaMemcpyAsync(f->host_result.as<double>() + 5, f->result.as<double>() + 5, sizeof(double),
                                   cudaMemcpyDeviceToHost, f->stream), "correlation readback");
        check_cuda(cudaStreamSynchronize(f->stream), "overlap correlation");
        const double peak = r[0], mean = r[3], sd = r[4];
        out[0] = dx;
        out[1] = dy;
        out[2] = (peak - mean) / (sd > 1e-12 ? sd : 1e-12);
        const double ox = (double)(n - abs(dx) > 0 ? n - abs(dx) : 0), oy = (double)(n - abs(dy) > 0 ? n - abs(dy) : 0);
        out[3] = ox * oy / ((double)n * n);
        out[4] = r[5];
        out[5] = peak;
    });
}

int gbdic_fourier_shift_device(gbdic_fourier *f, const uint8_t *frame, int64_t row_stride, int32_t height, int32_t x,
                               int32_t y, float multiplier, float *rows, int32_t count, int32_t pitch, void *stream) {
    return fguarded(f, [&] {
        if (!frame || !rows || count < 0 || pitch < 4) fail(GBDIC_EINVAL, "frame, rows (pitch >= 4) and count >= 0 are required");
        const int n = f->size;
        if (row_stride < x + n || x < 0 || y < 0 || y + n > height) fail(GBDIC_EINVAL, "window outside the frame");
        // The caller's stream orders everything: the transform buffers belong
        // to this handle, so calls on one handle must not overlap.
        cudaStream_t s = static_cast<cudaStream_t>(stream);
        // Outside a stream capture the call is ordered after the handle's own
        // stream (host-path estimates) and before its later work; inside a
        // capture (a CUDA graph of the caller's frame) the graph's launches
        // are ordered by the caller, and the handle's stream stays out of it.
        cudaStreamCaptureStatus capture = cudaStreamCaptureStatusNone;
        check_cuda(cudaStreamIsCapturing(s, &capture), "capture query");
        const bool capturing = capture != cudaStreamCaptureStatusNone;
        if (!capturing) {
            check_cuda(cudaEventRecord(f->fork, f->stream), "event");
            check_cuda(cudaStreamWaitEvent(s, f->fork, 0), "event wait");
        }
        check_cuda(cudaMemcpy2DAsync(f->window.get(), n, frame + (size_t)y * row_stride + x, (size_t)row_stride, n, n,
                                     cudaMemcpyDeviceToDevice, s), "window copy");
        f->spectrum_of(f->window.as<uint8_t>(), nullptr, f->cur_samples.as<double>(), nullptr, s);
        const int px = n * n;
        cross_power_kernel<<<(px + 255) / 256, 256, 0, s>>>(f->work.as<double2>(), f->ref_spectrum.as<double2>(), px);
        check_cuda(cudaGetLastError(), "cross power");
        f->transform(+1.0, s);
        double *pb = f->partials.as<double>();
        peak_partial_kernel<<<kPeakCtas, kPeakThreads, 0, s>>>(f->work.as<double2>(), n, pb,
                                                               reinterpret_cast<int *>(pb + kPeakCtas),
                                                               pb + 2 * kPeakCtas, pb + 3 * kPeakCtas);
        check_cuda(cudaGetLastError(), "peak");
        peak_final_kernel<<<1, kPeakCtas, 0, s>>>(f->work.as<double2>(), n, pb,
                                                  reinterpret_cast<const int *>(pb + kPeakCtas), pb + 2 * kPeakCtas,
                                                  pb + 3 * kPeakCtas, f->result.as<double>());
        check_cuda(cudaGetLastError(), "peak");
        if (count > 0) {
            const int blocks = count < 256 * 64 ? (count + 255) / 256 : 64;
            shift_rows_kernel<<<blocks, 256, 0, s>>>(f->result.as<double>(), f->sums.as<unsigned long long>(), n,
                                                     multiplier, rows, count, pitch);
            check_cuda(cudaGetLastError(), "shift rows");
        }
        // Later host-path estimates on the handle's own stream wait for this one.
        if (!capturing) {
            check_cuda(cudaEventRecord(f->join, s), "event");
            check_cuda(cudaStreamWaitEvent(f->stream, f->join, 0), "event wait");
        }
    });
}

}  // extern "C"
