// Second-order kernels for 2 general direction(s) at once (epg_second.cuh);
// one translation unit per table so they compile in parallel.
#include "epg_second.cuh"

namespace tsg {

extern const SecondEntry kSecondK2[];
extern const int kSecondK2Count;

const SecondEntry kSecondK2[] = {
    TSG_SECOND_ENTRY(4, 1, 2, 0),
    TSG_SECOND_ENTRY(4, 2, 2, 0),
    TSG_SECOND_ENTRY(4, 4, 2, 0),
    TSG_SECOND_ENTRY(4, 5, 2, 0),
    TSG_SECOND_ENTRY(4, 8, 2, 0),
    TSG_SECOND_ENTRY(2, 5, 2, 0),
    TSG_SECOND_ENTRY(2, 10, 2, 0),
    TSG_SECOND_ENTRY(2, 16, 2, 0),
    TSG_SECOND_ENTRY(2, 32, 2, 0),
};
const int kSecondK2Count = int(sizeof(kSecondK2) / sizeof(kSecondK2[0]));

}  // namespace tsg
