// Compile-check stand-in for OpenMM's KernelImpl.
#pragma once
#include <string>
#include "openmm/internal/windowsExport.h"
namespace OpenMM {
class Platform;
class KernelImpl {
public:
    KernelImpl(std::string name, const Platform& platform);
    virtual ~KernelImpl();
};
}
