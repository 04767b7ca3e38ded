// Compile-check stand-in for OpenMM's export macro.
#pragma once
#define OPENMM_EXPORT __attribute__((visibility("default")))
