// Second-order kernels for the one-hot direction set T2 (epg_second.cuh,
// direction code 2); one translation unit per set so they compile in
// parallel.
#include "epg_second.cuh"

namespace tsg {

extern const SecondEntry kSecondHotT2[];
extern const int kSecondHotT2Count;

const SecondEntry kSecondHotT2[] = {TSG_SECOND_SHAPES_HOT(1, 2)};
const int kSecondHotT2Count = int(sizeof(kSecondHotT2) / sizeof(kSecondHotT2[0]));

}  // namespace tsg
