// Minimal stand-in for the parts of OpenMM's System that the rigid-body plugin's CPU code reads:
// particle masses, the virtual-site flag and the constraint list (oracle test infrastructure only).
#ifndef RBX_STANDIN_SYSTEM_H
#define RBX_STANDIN_SYSTEM_H
#include <vector>
namespace OpenMM {
class System {
public:
    int addParticle(double mass) { masses.push_back(mass); virt.push_back(false); return (int)masses.size() - 1; }
    int getNumParticles() const { return (int)masses.size(); }
    double getParticleMass(int i) const { return masses[i]; }
    bool isVirtualSite(int i) const { return virt[i]; }
    void setVirtualSite(int i, bool flag) { virt[i] = flag; }
    int addConstraint(int a, int b, double dist) { ca.push_back(a); cb.push_back(b); cd.push_back(dist); return (int)ca.size() - 1; }
    int getNumConstraints() const { return (int)ca.size(); }
    void getConstraintParameters(int i, int& a, int& b, double& dist) const { a = ca[i]; b = cb[i]; dist = cd[i]; }
private:
    std::vector<double> masses;
    std::vector<bool> virt;
    std::vector<int> ca, cb;
    std::vector<double> cd;
};
}  // namespace OpenMM
#endif
