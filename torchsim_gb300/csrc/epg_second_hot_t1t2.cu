// Second-order kernels for the one-hot direction set T1T2 (epg_second.cuh,
// direction code 9); one translation unit per set so they compile in
// parallel.
#include "epg_second.cuh"

namespace tsg {

extern const SecondEntry kSecondHotT1T2[];
extern const int kSecondHotT1T2Count;

const SecondEntry kSecondHotT1T2[] = {TSG_SECOND_SHAPES_HOT(2, 9)};
const int kSecondHotT1T2Count = int(sizeof(kSecondHotT1T2) / sizeof(kSecondHotT1T2[0]));

}  // namespace tsg
