// Compile-check stand-in for OpenMM's Platform.
#pragma once
#include <string>
#include "openmm/internal/windowsExport.h"
namespace OpenMM {
class KernelFactory;
class Platform {
public:
    static Platform& getPlatformByName(const std::string& name);
    void registerKernelFactory(const std::string& name, KernelFactory* factory);
};
}
