// Second-order kernels for the one-hot direction set T1B1 (epg_second.cuh,
// direction code 13); one translation unit per set so they compile in
// parallel.
#include "epg_second.cuh"

namespace tsg {

extern const SecondEntry kSecondHotT1B1[];
extern const int kSecondHotT1B1Count;

const SecondEntry kSecondHotT1B1[] = {TSG_SECOND_SHAPES_HOT(2, 13)};
const int kSecondHotT1B1Count = int(sizeof(kSecondHotT1B1) / sizeof(kSecondHotT1B1[0]));

}  // namespace tsg
