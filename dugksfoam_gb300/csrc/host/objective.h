// Gradient harness of the FP64 step (objective.cpp): a wall-flux objective
// over a window of steps from the initial state, its tangent-linear
// directional derivative and its adjoint gradient with respect to the wall
// temperatures T_w (every wall face) and the viscosity scale s (mu_ref -> s mu_ref,
// derivative at s = 1).
//
//   J = 1/(n_steps - avg_first) * sum_{n = avg_first}^{n_steps-1}
//         [ sum_{w in q_patch} S_w . qWall_w(n)  +  sum_{w in stress_patch} |S_w| stressWall_w,xy(n) ]
//
// qWall, stressWall as fvDVM::updateMacroSurf forms them (fvDVM.C:535-576).
// The forward is the plain FP64 reference pipeline on private buffers; the
// handle's own state is not touched.
#pragma once

#include "solver.h"

namespace dugks {

struct Objective {
    int nSteps = 0, avgFirst = 0;
    int qPatch = -1, stressPatch = -1;
    int ckptEvery = 1;
};

int objective_value(Solver& s, const Objective& o, double& J);
int objective_tangent(Solver& s, const Objective& o, const double* dTw, double dMuScale, double& J, double& dJ);
int objective_adjoint(Solver& s, const Objective& o, double& J, double* dJdTw, double& dJdMuScale);

}  // namespace dugks
