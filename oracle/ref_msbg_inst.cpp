/*
 * The reference's src/msbg.cpp, compiled as it lies, plus one explicit template
 * instantiation the release never makes: MultiresSparseGrid::dotProdChannel_<float>
 * (src/msbg.cpp:4524-4646) has no caller in the library, so no object file holds it,
 * and the oracle's solver job calls it through dotProdChannel (src/msbg.h:3333-3341).
 * Test infrastructure only.
 */
#include "msbg.cpp"

namespace MSBG {
template long double MultiresSparseGrid::dotProdChannel_<float>(int, int, int, std::vector<int> *, int *);
}
