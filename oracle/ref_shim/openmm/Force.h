/* Oracle build shim (test infrastructure only): just enough of OpenMM's Force base
 * class for openmm/MPIDForce.h to parse; nothing from MPIDForce.cpp is linked. */
#ifndef MPID_ORACLE_SHIM_FORCE_H
#define MPID_ORACLE_SHIM_FORCE_H
#include <string>
namespace OpenMM {
class Context;
class ForceImpl;
class Force {
public:
    Force() : forceGroup(0) {}
    virtual ~Force() {}
    int getForceGroup() const { return forceGroup; }
    void setForceGroup(int g) { forceGroup = g; }
    virtual bool usesPeriodicBoundaryConditions() const { return false; }
protected:
    virtual ForceImpl* createImpl() const = 0;
    ForceImpl& getImplInContext(Context& context);
    const ForceImpl& getImplInContext(const Context& context) const;
private:
    int forceGroup;
};
}
#endif
