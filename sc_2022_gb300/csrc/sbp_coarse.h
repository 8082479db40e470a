// Dense inverse of the re-discretised coarse operator (host, cached).
#pragma once

#include <memory>
#include <vector>

namespace sbp {

// Row-major (= column-major, it is symmetric) nc^2 x nc^2 inverse of A on an
// nc x nc grid.  Throws std::runtime_error if the factorisation fails.
std::shared_ptr<const std::vector<double>> coarse_inverse(int nc);

}  // namespace sbp
