/* Oracle build shim (test infrastructure only).
 * Interface of the 3-D complex FFT that the reference's CPU PME code calls
 * (platforms/reference/src/SimTKReference/MPIDReferenceForce.cpp:2604-2606, 2931-2933,
 * 4066-4068).  The implementation is oracle/fft3d.cpp: an unnormalised mixed-radix
 * transform, exp(-i...) forward and exp(+i...) backward. */
#ifndef MPID_ORACLE_SHIM_FFTPACK_H
#define MPID_ORACLE_SHIM_FFTPACK_H
struct t_complex {
    double re, im;
    t_complex() : re(0.0), im(0.0) {}
    t_complex(double r, double i) : re(r), im(i) {}
};
struct fftpack;
typedef struct fftpack* fftpack_t;
typedef enum { FFTPACK_FORWARD = 0, FFTPACK_BACKWARD = 1 } fftpack_direction;
int fftpack_init_3d(fftpack_t* plan, int nx, int ny, int nz);
int fftpack_exec_3d(fftpack_t plan, fftpack_direction dir, t_complex* in, t_complex* out);
void fftpack_destroy(fftpack_t plan);
#endif
