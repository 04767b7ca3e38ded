// Compile-check stand-in for OpenMM's OpenMMException.
#pragma once
#include <stdexcept>
#include <string>
namespace OpenMM {
class OpenMMException : public std::runtime_error {
public:
    explicit OpenMMException(const std::string& m) : std::runtime_error(m) {}
};
}
