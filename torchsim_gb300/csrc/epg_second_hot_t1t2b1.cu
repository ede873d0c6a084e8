// Second-order kernels for the one-hot direction set T1T2B1 (epg_second.cuh,
// direction code 57); one translation unit per set so they compile in
// parallel.
#include "epg_second.cuh"

namespace tsg {

extern const SecondEntry kSecondHotT1T2B1[];
extern const int kSecondHotT1T2B1Count;

const SecondEntry kSecondHotT1T2B1[] = {TSG_SECOND_SHAPES_HOT(3, 57)};
const int kSecondHotT1T2B1Count = int(sizeof(kSecondHotT1T2B1) / sizeof(kSecondHotT1T2B1[0]));

}  // namespace tsg
