// Minimal stand-in for OpenMM's exception type (test infrastructure for the oracle only).
#ifndef RBX_STANDIN_OPENMMEXCEPTION_H
#define RBX_STANDIN_OPENMMEXCEPTION_H
#include <stdexcept>
#include <string>
namespace OpenMM {
class OpenMMException : public std::runtime_error {
public:
    explicit OpenMMException(const std::string& msg) : std::runtime_error(msg) {}
};
}  // namespace OpenMM
#endif
