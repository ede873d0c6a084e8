// Second-order kernels for the one-hot direction set B1 (epg_second.cuh,
// direction code 3); one translation unit per set so they compile in
// parallel.
#include "epg_second.cuh"

namespace tsg {

extern const SecondEntry kSecondHotB1[];
extern const int kSecondHotB1Count;

const SecondEntry kSecondHotB1[] = {TSG_SECOND_SHAPES_HOT(1, 3)};
const int kSecondHotB1Count = int(sizeof(kSecondHotB1) / sizeof(kSecondHotB1[0]));

}  // namespace tsg
