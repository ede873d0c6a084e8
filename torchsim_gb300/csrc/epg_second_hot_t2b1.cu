// Second-order kernels for the one-hot direction set T2B1 (epg_second.cuh,
// direction code 14); one translation unit per set so they compile in
// parallel.
#include "epg_second.cuh"

namespace tsg {

extern const SecondEntry kSecondHotT2B1[];
extern const int kSecondHotT2B1Count;

const SecondEntry kSecondHotT2B1[] = {TSG_SECOND_SHAPES_HOT(2, 14)};
const int kSecondHotT2B1Count = int(sizeof(kSecondHotT2B1) / sizeof(kSecondHotT2B1[0]));

}  // namespace tsg
