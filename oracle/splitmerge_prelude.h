// splitmerge_prelude.h -- TEST INFRASTRUCTURE ONLY.
//
// Streamed by oracle/build_ref.sh ahead of the reference's Split.h and Merge.h (each cut
// before its *_operation wrapper, which needs the element classes).  The Eigen matrix
// comes from oracle/eigen_shim; Omega3D.h (Dimensions, numStrPerNode) is the reference's.
#pragma once
#include <Eigen/Dense>
#include "Omega3D.h"
