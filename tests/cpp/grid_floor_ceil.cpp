// ctypes shim over wide_grid_floor_ceil (bvh_boxes.h) for the exactness test in
// tests/test_wide_bvh.py: n planes v against grid origins org and power-of-two inverses inv.
#include "bvh_boxes.h"

extern "C" void grid_floor_ceil(float const *v, float const *org, float const *inv, int n, float *fl, float *cl) {
    for (int k = 0; k < n; k++)
        e8g::wide_grid_floor_ceil(v[k], org[k], inv[k], fl[k], cl[k]);
}
