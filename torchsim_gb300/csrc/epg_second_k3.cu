// Second-order kernels for 3 general direction(s) at once (epg_second.cuh);
// one translation unit per table so they compile in parallel.
#include "epg_second.cuh"

namespace tsg {

extern const SecondEntry kSecondK3[];
extern const int kSecondK3Count;

const SecondEntry kSecondK3[] = {
    TSG_SECOND_ENTRY(4, 1, 3, 0),
    TSG_SECOND_ENTRY(4, 2, 3, 0),
    TSG_SECOND_ENTRY(4, 4, 3, 0),
    TSG_SECOND_ENTRY(4, 5, 3, 0),
    TSG_SECOND_ENTRY(4, 8, 3, 0),
    TSG_SECOND_ENTRY(2, 5, 3, 0),
    TSG_SECOND_ENTRY(2, 10, 3, 0),
    TSG_SECOND_ENTRY(2, 16, 3, 0),
    TSG_SECOND_ENTRY(2, 32, 3, 0),
};
const int kSecondK3Count = int(sizeof(kSecondK3) / sizeof(kSecondK3[0]));

}  // namespace tsg
