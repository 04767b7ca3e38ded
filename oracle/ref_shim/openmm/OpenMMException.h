/* Oracle build shim (test infrastructure only): the exception type the reference's
 * CPU force throws on non-convergence and invalid boxes. */
#ifndef MPID_ORACLE_SHIM_EXCEPTION_H
#define MPID_ORACLE_SHIM_EXCEPTION_H
#include <exception>
#include <string>
#include <sstream>
namespace OpenMM {
class OpenMMException : public std::exception {
public:
    explicit OpenMMException(const std::string& m) : msg(m) {}
    ~OpenMMException() throw() {}
    const char* what() const throw() { return msg.c_str(); }
private:
    std::string msg;
};
}
#endif
