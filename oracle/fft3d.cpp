/* Oracle support code (test infrastructure only; never linked into the product).
 *
 * Double-precision 3-D complex FFT behind the fftpack interface that the reference's
 * CPU PME force uses (MPIDReferenceForce.cpp:2604-2606 plan, :2931/:2933 and
 * :4066/:4068 execute).  OpenMM's fftpack is not available here, so this is a plain
 * mixed-radix Cooley-Tukey transform applied along each axis of a row-major
 * (x slowest, z fastest) grid.  Convention: forward uses exp(-2 pi i jk/n), backward
 * exp(+2 pi i jk/n), neither direction is normalised; the reference's reciprocal
 * convolution carries the 1/(pi V) factor itself (MPIDReferenceForce.cpp:3333).
 */
#include "fftpack.h"
#include <cmath>
#include <complex>
#include <vector>

typedef std::complex<double> cplx;

struct fftpack {
    int n[3];
    std::vector<cplx> tw[3];   // exp(-2 pi i k / n) for k < n, per axis
};

static void make_twiddles(std::vector<cplx>& tw, int n) {
    tw.resize(n);
    for (int k = 0; k < n; ++k) {
        // Angles reduced to the first octant-free exact form: 2 pi k / n.
        double a = -2.0 * M_PI * (double) k / (double) n;
        tw[k] = cplx(cos(a), sin(a));
    }
}

/* Recursive decimation-in-time transform of `in` (stride s, length n) into `out`
 * (contiguous).  `tw` holds the length-N root table; `step` = N/n selects roots. */
static void fft_rec(const cplx* in, int s, int n, cplx* out, const std::vector<cplx>& tw, int step,
                    bool inverse, std::vector<cplx>& scratch) {
    if (n == 1) {
        out[0] = in[0];
        return;
    }
    int p = 2;
    while (p * p <= n && n % p != 0)
        ++p;
    if (n % p != 0)
        p = n;  // n is prime
    int m = n / p;
    int N = (int) tw.size();
    if (m == 1) {
        // Direct DFT of a prime length.
        for (int k = 0; k < n; ++k) {
            cplx acc(0.0, 0.0);
            for (int j = 0; j < n; ++j) {
                long idx = ((long) j * k % n) * step;
                cplx w = tw[idx % N];
                if (inverse) w = std::conj(w);
                acc += in[(long) j * s] * w;
            }
            out[k] = acc;
        }
        return;
    }
    // p sub-transforms of length m over the residues r = 0..p-1.
    std::vector<cplx> sub((size_t) n);
    for (int r = 0; r < p; ++r)
        fft_rec(in + (long) r * s, s * p, m, sub.data() + (size_t) r * m, tw, step * p, inverse, scratch);
    // Combine: X[k + q m] = sum_r W_n^{r (k + q m)} Y_r[k].
    for (int k = 0; k < m; ++k) {
        for (int q = 0; q < p; ++q) {
            int kk = k + q * m;
            cplx acc(0.0, 0.0);
            for (int r = 0; r < p; ++r) {
                long idx = ((long) r * kk % n) * step;
                cplx w = tw[idx % N];
                if (inverse) w = std::conj(w);
                acc += sub[(size_t) r * m + k] * w;
            }
            out[kk] = acc;
        }
    }
}

int fftpack_init_3d(fftpack_t* plan, int nx, int ny, int nz) {
    if (nx <= 0 || ny <= 0 || nz <= 0)
        return -1;
    fftpack* f = new fftpack;
    f->n[0] = nx;
    f->n[1] = ny;
    f->n[2] = nz;
    for (int d = 0; d < 3; ++d)
        make_twiddles(f->tw[d], f->n[d]);
    *plan = f;
    return 0;
}

int fftpack_exec_3d(fftpack_t plan, fftpack_direction dir, t_complex* in, t_complex* out) {
    const int nx = plan->n[0], ny = plan->n[1], nz = plan->n[2];
    const bool inverse = (dir == FFTPACK_BACKWARD);
    const long total = (long) nx * ny * nz;
    std::vector<cplx> grid((size_t) total);
    for (long i = 0; i < total; ++i)
        grid[i] = cplx(in[i].re, in[i].im);
    std::vector<cplx> line, res, scratch;
    const int dims[3] = {nx, ny, nz};
    const long strides[3] = {(long) ny * nz, (long) nz, 1};
    for (int d = 0; d < 3; ++d) {
        int n = dims[d];
        line.resize(n);
        res.resize(n);
        // Iterate over all lines along axis d.
        for (int a = 0; a < dims[(d + 1) % 3]; ++a) {
            for (int b = 0; b < dims[(d + 2) % 3]; ++b) {
                long base = (long) a * strides[(d + 1) % 3] + (long) b * strides[(d + 2) % 3];
                for (int k = 0; k < n; ++k)
                    line[k] = grid[base + (long) k * strides[d]];
                fft_rec(line.data(), 1, n, res.data(), plan->tw[d], 1, inverse, scratch);
                for (int k = 0; k < n; ++k)
                    grid[base + (long) k * strides[d]] = res[k];
            }
        }
    }
    for (long i = 0; i < total; ++i) {
        out[i].re = grid[i].real();
        out[i].im = grid[i].imag();
    }
    return 0;
}

void fftpack_destroy(fftpack_t plan) { delete plan; }
