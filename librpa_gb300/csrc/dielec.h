// The macroscopic dielectric function eps(i omega) on the minimax frequencies, for the head
// correction of W at q = 0: LibRPA's interpolate_dielec_func (src/core/dielecmodel.cpp:65-104).
// Host work on a few dozen numbers, as in the reference.
#pragma once

#include <vector>

namespace gb {

// option 0: the input values unchanged (the input grid must be the target grid);
// option 1: natural cubic spline through the input points, evaluated at the targets
//           (src/math/interpolate.cpp:9-150);
// option 2: least-squares fit of the two-term Havriliak-Negami model
//           1 + (e1 - 1) / (1 + (u t1)^a1)^b1 + (e2 - 1) / (1 + (u t2)^a2)^b2
//           by Levenberg-Marquardt (src/math/fitting.cpp:99-199, dielecmodel.cpp:34-63),
//           evaluated at the targets.
std::vector<double> interpolate_dielec_func(int option, const std::vector<double> &omega_in,
                                            const std::vector<double> &eps_in,
                                            const std::vector<double> &omega_target);

} // namespace gb
