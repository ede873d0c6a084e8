// Second-order kernels for 2 direction(s) at once (epg_second.cuh), one
// translation unit per direction count so they compile in parallel.
#include "epg_second.cuh"

namespace tsg {

extern const SecondEntry kSecondK2[];
extern const int kSecondK2Count;

const SecondEntry kSecondK2[] = {
    TSG_SECOND_ENTRY(4, 1, 2), TSG_SECOND_ENTRY(4, 2, 2), TSG_SECOND_ENTRY(4, 3, 2),
    TSG_SECOND_ENTRY(4, 4, 2), TSG_SECOND_ENTRY(4, 5, 2), TSG_SECOND_ENTRY(4, 8, 2),
    TSG_SECOND_ENTRY(4, 16, 2),
};
const int kSecondK2Count = int(sizeof(kSecondK2) / sizeof(kSecondK2[0]));

}  // namespace tsg
