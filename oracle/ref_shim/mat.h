// TEST INFRASTRUCTURE ONLY.  Empty stand-in for MATLAB's mat.h, which the
// reference's include/quantum/QuantumOperator.h includes; the pinned code
// writes no MAT-files (its export is compiled without HAS_MATLAB).
#pragma once
