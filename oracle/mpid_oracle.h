/* Oracle C interface (test infrastructure only).
 *
 * One plain-C entry point per oracle build: `mpidref_evaluate` (the reference's own
 * FP64 CPU force, compiled in place into oracle/_ref/) and `mpidport_evaluate` (this
 * directory's C restatement, mpid_port.c).  Both take the same flat description of an
 * MPIDForce system, mirroring what ReferenceCalcMPIDForceKernel::initialize copies out
 * of an MPIDForce (platforms/reference/src/MPIDReferenceKernels.cpp:84-177), and return
 * energy, forces and dipoles.  Only tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline may load these libraries.
 *
 * Units: nm, e, kJ/mol.  Parameter orders follow MPIDForce::addMultipole:
 *   dipole      X Y Z
 *   quadrupole  XX XY YY XZ YZ ZZ
 *   octopole    XXX XXY XYY YYY XXZ XYZ YYZ XZZ YZZ ZZZ
 */
#ifndef MPID_ORACLE_H
#define MPID_ORACLE_H
#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    int n;                      /* number of atoms */
    const double* pos;          /* 3n */
    const double* charge;       /* n */
    const double* dipole;       /* 3n, molecular frame */
    const double* quadrupole;   /* 6n, molecular frame */
    const double* octopole;     /* 10n, molecular frame */
    const double* thole;        /* n */
    const double* polarity;     /* 3n, molecular-frame diagonal */
    const int* axis_type;       /* n: 0 ZThenX 1 Bisector 2 ZBisect 3 ThreeFold 4 ZOnly 5 NoAxisType */
    const int* atom_z;          /* n */
    const int* atom_x;          /* n */
    const int* atom_y;          /* n */
    const int* cov_offsets;     /* 8n+1: CSR offsets over (atom, covalent type) */
    const int* cov_index;       /* cov_offsets[8n] entries */
    int nonbonded_method;       /* 0 NoCutoff, 1 PME */
    int polarization_type;      /* 0 Mutual, 1 Direct, 2 Extrapolated */
    double cutoff;              /* nm */
    double ewald_alpha;         /* nm^-1 */
    int grid[3];
    int pme_order;              /* port: 5 or 6; the reference build is fixed at 6 */
    double box[9];              /* row vectors a, b, c */
    double mutual_eps;          /* Debye */
    int max_iter;
    int n_extrap;
    const double* extrap_coeffs;
    double default_thole;
    double scale14;
} mpid_oracle_input;

typedef struct {
    double energy;              /* kJ/mol */
    double* forces;             /* 3n, overwritten */
    double* induced;            /* 3n or NULL: induced dipoles, e nm */
    double* labdipoles;         /* 3n or NULL: lab-frame permanent dipoles, e nm */
    int iterations;
    double epsilon;             /* final Debye RMS residual (Mutual) */
    int converged;
    char message[512];
    double* grad;               /* 20n or NULL (port only): dE/d(molecular-frame charge, dipole X Y Z,
                                   quadrupole XX XY YY XZ YZ ZZ, octopole XXX ... ZZZ) per atom */
    double* polgrad;            /* 4n or NULL (port only): dE/d(molecular-frame
                                   polarisability X Y Z, Thole width) per atom */
} mpid_oracle_output;

int mpidref_evaluate(const mpid_oracle_input* in, mpid_oracle_output* out);
int mpidref_properties(const mpid_oracle_input* in, const double* masses, const double* grid, int ngrid,
                       double* moments, double* potential, char* message);
int mpidport_evaluate(const mpid_oracle_input* in, mpid_oracle_output* out);

#ifdef __cplusplus
}
#endif
#endif
