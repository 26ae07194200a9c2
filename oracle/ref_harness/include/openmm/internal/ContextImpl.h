// Minimal stand-in for OpenMM's ContextImpl: it hands the plugin's CPU code a System and the
// current positions, velocities and forces held in host arrays (oracle test infrastructure only).
#ifndef RBX_STANDIN_CONTEXTIMPL_H
#define RBX_STANDIN_CONTEXTIMPL_H
#include "openmm/System.h"
#include "openmm/Vec3.h"
#include <vector>
namespace OpenMM {
class ContextImpl {
public:
    explicit ContextImpl(const System& s) : sys(s) {}
    const System& getSystem() const { return sys; }
    void getPositions(std::vector<Vec3>& out) { out = positions; }
    void getVelocities(std::vector<Vec3>& out) { out = velocities; }
    void getForces(std::vector<Vec3>& out) { out = forces; }
    std::vector<Vec3> positions, velocities, forces;
private:
    const System& sys;
};
}  // namespace OpenMM
#endif
