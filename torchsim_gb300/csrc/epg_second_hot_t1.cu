// Second-order kernels for the one-hot direction set T1 (epg_second.cuh,
// direction code 1); one translation unit per set so they compile in
// parallel.
#include "epg_second.cuh"

namespace tsg {

extern const SecondEntry kSecondHotT1[];
extern const int kSecondHotT1Count;

const SecondEntry kSecondHotT1[] = {TSG_SECOND_SHAPES_HOT(1, 1)};
const int kSecondHotT1Count = int(sizeof(kSecondHotT1) / sizeof(kSecondHotT1[0]));

}  // namespace tsg
