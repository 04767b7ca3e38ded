/* Oracle driver for the reference's own FP64 CPU force (test infrastructure only).
 *
 * Compiled together with platforms/reference/src/SimTKReference/MPIDReferenceForce.cpp,
 * unmodified and in place, by oracle/Makefile; the output lands in oracle/_ref/.  This
 * file plays the part of ReferenceCalcMPIDForceKernel (MPIDReferenceKernels.cpp):
 *   - initialize():            flat parameter copy, dampingFactor = (mean alpha)^(1/6)
 *                              (MPIDReferenceKernels.cpp:84-177, :126)
 *   - setupMPIDReferenceForce: PME or NoCutoff object, alpha/cutoff/grid/box, the
 *                              box >= 1.999999 cutoff check, solver settings, 1-4 scale
 *                              (MPIDReferenceKernels.cpp:179-223)
 *   - execute():               calculateForceAndEnergy (MPIDReferenceKernels.cpp:225-239)
 * OpenMM's Context is absent, so explicit PME parameters are required (no
 * NonbondedForceImpl::calcPMEParameters fallback, MPIDReferenceKernels.cpp:161-170).
 */
#include "MPIDReferenceForce.h"
#include "mpid_oracle.h"
#include <cstring>
#include <cstdio>
#include <exception>

using namespace OpenMM;

namespace {

// Exposes the protected induced dipoles after calculateForceAndEnergy() ran setup().
class TappedPme : public MPIDReferencePmeForce {
public:
    const std::vector<Vec3>& induced() const { return _inducedDipole; }
};
class TappedNoCut : public MPIDReferenceForce {
public:
    TappedNoCut() : MPIDReferenceForce(MPIDReferenceForce::NoCutoff) {}
    const std::vector<Vec3>& induced() const { return _inducedDipole; }
};

void configure(MPIDReferenceForce* f, const mpid_oracle_input* in) {
    f->setDefaultTholeWidth(in->default_thole);
    if (in->polarization_type == 0) {
        f->setPolarizationType(MPIDReferenceForce::Mutual);
        f->setMutualInducedDipoleTargetEpsilon(in->mutual_eps);
        f->setMaximumMutualInducedDipoleIterations(in->max_iter);
    } else if (in->polarization_type == 1) {
        f->setPolarizationType(MPIDReferenceForce::Direct);
    } else if (in->polarization_type == 2) {
        f->setPolarizationType(MPIDReferenceForce::Extrapolated);
        std::vector<double> c(in->extrap_coeffs, in->extrap_coeffs + in->n_extrap);
        f->setExtrapolationCoefficients(c);
    } else {
        throw OpenMMException("Polarization type not recognzied.");
    }
    f->set14ScaleFactor(in->scale14);
}

// The flat oracle input unpacked into the reference's argument vectors.
struct Unpacked {
    int n;
    std::vector<Vec3> pos;
    std::vector<double> charges, dipoles, quads, octs, tholes, damp;
    std::vector<std::vector<double> > polarity;
    std::vector<int> axis, az, ax, ay;
    std::vector<std::vector<std::vector<int> > > cov;
    explicit Unpacked(const mpid_oracle_input* in) : n(in->n) {
        pos.resize(n);
        charges.resize(n); dipoles.resize(3 * n); quads.resize(6 * n); octs.resize(10 * n); tholes.resize(n);
        damp.resize(n); polarity.resize(n); axis.resize(n); az.resize(n); ax.resize(n); ay.resize(n); cov.resize(n);
        for (int i = 0; i < n; ++i) {
            pos[i] = Vec3(in->pos[3 * i], in->pos[3 * i + 1], in->pos[3 * i + 2]);
            charges[i] = in->charge[i];
            for (int k = 0; k < 3; ++k) dipoles[3 * i + k] = in->dipole[3 * i + k];
            for (int k = 0; k < 6; ++k) quads[6 * i + k] = in->quadrupole[6 * i + k];
            for (int k = 0; k < 10; ++k) octs[10 * i + k] = in->octopole[10 * i + k];
            tholes[i] = in->thole[i];
            polarity[i] = std::vector<double>(in->polarity + 3 * i, in->polarity + 3 * i + 3);
            damp[i] = pow((polarity[i][0] + polarity[i][1] + polarity[i][2]) / 3.0, 1.0 / 6.0);
            axis[i] = in->axis_type[i];
            az[i] = in->atom_z[i];
            ax[i] = in->atom_x[i];
            ay[i] = in->atom_y[i];
            cov[i].resize(8);
            for (int t = 0; t < 8; ++t)
                for (int k = in->cov_offsets[8 * i + t]; k < in->cov_offsets[8 * i + t + 1]; ++k)
                    cov[i][t].push_back(in->cov_index[k]);
        }
    }
};

// PME or no-cutoff reference force configured as setupMPIDReferenceForce does.
MPIDReferenceForce* make_force(const mpid_oracle_input* in) {
    MPIDReferenceForce* base = nullptr;
    if (in->nonbonded_method == 1) {
        TappedPme* pme = new TappedPme();
        pme->setAlphaEwald(in->ewald_alpha);
        pme->setCutoffDistance(in->cutoff);
        std::vector<int> grid(in->grid, in->grid + 3);
        pme->setPmeGridDimensions(grid);
        Vec3 box[3] = {Vec3(in->box[0], in->box[1], in->box[2]), Vec3(in->box[3], in->box[4], in->box[5]),
                       Vec3(in->box[6], in->box[7], in->box[8])};
        pme->setPeriodicBoxSize(box);
        base = pme;
    } else {
        base = new TappedNoCut();
    }
    configure(base, in);
    return base;
}

}  // namespace

/* getSystemMultipoleMoments and getElectrostaticPotential of the reference kernel
 * (MPIDReferenceKernels.cpp:302-341): 13 moments for the given masses, and the potential
 * (kJ/mol/e) at ngrid points (3 doubles each). */
extern "C" int mpidref_properties(const mpid_oracle_input* in, const double* masses, const double* grid, int ngrid,
                                  double* moments, double* potential, char* message) {
    message[0] = 0;
    try {
        Unpacked u(in);
        std::vector<double> m(masses, masses + in->n);
        std::vector<double> mom;
        MPIDReferenceForce* f = make_force(in);
        f->calculateMPIDSystemMultipoleMoments(m, u.pos, u.charges, u.dipoles, u.quads, u.octs, u.tholes, u.damp,
                                               u.polarity, u.axis, u.az, u.ax, u.ay, u.cov, mom);
        for (int k = 0; k < 13; ++k) moments[k] = mom[k];
        std::vector<Vec3> g(ngrid);
        for (int k = 0; k < ngrid; ++k) g[k] = Vec3(grid[3 * k], grid[3 * k + 1], grid[3 * k + 2]);
        std::vector<double> pot;
        f->calculateElectrostaticPotential(u.pos, u.charges, u.dipoles, u.quads, u.octs, u.tholes, u.damp, u.polarity,
                                           u.axis, u.az, u.ax, u.ay, u.cov, g, pot);
        for (int k = 0; k < ngrid; ++k) potential[k] = pot[k];
        delete f;
        return 0;
    } catch (const std::exception& e) {
        snprintf(message, 512, "%s", e.what());
        return 1;
    }
}

extern "C" int mpidref_evaluate(const mpid_oracle_input* in, mpid_oracle_output* out) {
    out->message[0] = 0;
    try {
        const int n = in->n;
        std::vector<Vec3> pos(n);
        std::vector<double> charges(n), dipoles(3 * n), quads(6 * n), octs(10 * n), tholes(n), damp(n);
        std::vector<std::vector<double> > polarity(n);
        std::vector<int> axis(n), az(n), ax(n), ay(n);
        std::vector<std::vector<std::vector<int> > > cov(n);
        for (int i = 0; i < n; ++i) {
            pos[i] = Vec3(in->pos[3 * i], in->pos[3 * i + 1], in->pos[3 * i + 2]);
            charges[i] = in->charge[i];
            for (int k = 0; k < 3; ++k) dipoles[3 * i + k] = in->dipole[3 * i + k];
            for (int k = 0; k < 6; ++k) quads[6 * i + k] = in->quadrupole[6 * i + k];
            for (int k = 0; k < 10; ++k) octs[10 * i + k] = in->octopole[10 * i + k];
            tholes[i] = in->thole[i];
            polarity[i] = std::vector<double>(in->polarity + 3 * i, in->polarity + 3 * i + 3);
            damp[i] = pow((polarity[i][0] + polarity[i][1] + polarity[i][2]) / 3.0, 1.0 / 6.0);
            axis[i] = in->axis_type[i];
            az[i] = in->atom_z[i];
            ax[i] = in->atom_x[i];
            ay[i] = in->atom_y[i];
            cov[i].resize(8);
            for (int t = 0; t < 8; ++t)
                for (int k = in->cov_offsets[8 * i + t]; k < in->cov_offsets[8 * i + t + 1]; ++k)
                    cov[i][t].push_back(in->cov_index[k]);
        }
        std::vector<Vec3> forces(n, Vec3());
        double energy = 0.0;
        std::vector<Vec3> induced;
        MPIDReferenceForce* base = nullptr;
        TappedPme* pme = nullptr;
        TappedNoCut* nocut = nullptr;
        if (in->nonbonded_method == 1) {
            pme = new TappedPme();
            pme->setAlphaEwald(in->ewald_alpha);
            pme->setCutoffDistance(in->cutoff);
            std::vector<int> grid(in->grid, in->grid + 3);
            pme->setPmeGridDimensions(grid);
            Vec3 box[3] = {Vec3(in->box[0], in->box[1], in->box[2]), Vec3(in->box[3], in->box[4], in->box[5]),
                           Vec3(in->box[6], in->box[7], in->box[8])};
            double minAllowedSize = 1.999999 * in->cutoff;
            if (box[0][0] < minAllowedSize || box[1][1] < minAllowedSize || box[2][2] < minAllowedSize)
                throw OpenMMException("The periodic box size has decreased to less than twice the nonbonded cutoff.");
            pme->setPeriodicBoxSize(box);
            base = pme;
        } else {
            nocut = new TappedNoCut();
            base = nocut;
        }
        configure(base, in);
        try {
            energy = base->calculateForceAndEnergy(pos, charges, dipoles, quads, octs, tholes, damp, polarity, axis, az, ax,
                                                   ay, cov, forces);
        } catch (...) {
            out->iterations = base->getMutualInducedDipoleIterations();
            out->epsilon = base->getMutualInducedDipoleEpsilon();
            out->converged = base->getMutualInducedDipoleConverged();
            delete base;
            throw;
        }
        induced = pme ? pme->induced() : nocut->induced();
        out->energy = energy;
        for (int i = 0; i < n; ++i)
            for (int k = 0; k < 3; ++k) out->forces[3 * i + k] = forces[i][k];
        if (out->induced)
            for (int i = 0; i < n; ++i)
                for (int k = 0; k < 3; ++k) out->induced[3 * i + k] = induced[i][k];
        out->iterations = base->getMutualInducedDipoleIterations();
        out->epsilon = base->getMutualInducedDipoleEpsilon();
        out->converged = base->getMutualInducedDipoleConverged();
        if (out->labdipoles) {
            std::vector<Vec3> lab;
            base->calculateLabFramePermanentDipoles(pos, charges, dipoles, quads, octs, tholes, damp, polarity, axis, az, ax,
                                                    ay, cov, lab);
            for (int i = 0; i < n; ++i)
                for (int k = 0; k < 3; ++k) out->labdipoles[3 * i + k] = lab[i][k];
        }
        delete base;
        return 0;
    } catch (const std::exception& e) {
        snprintf(out->message, sizeof(out->message), "%s", e.what());
        return 1;
    }
}
