// fd_weights.cuh -- second-derivative weights shared by the 2-D and 3-D engines.
#pragma once

namespace gbfwi {

// Second-derivative weights of fd_coefficient (fdtd2D_modelling.c:1292-1325)
// for half-width H = Lc-1: the reference's double literals rounded to float,
// as compile-time constants (with m known at compile time they become
// instruction immediates).
template <int H>
__host__ __device__ constexpr float fd_weight(int m)
{
    if (H == 3) {
        return m == 0 ? (float)(-49.0 / 18) : m == 1 ? 1.5f : m == 2 ? (float)(-3.0 / 20) : (float)(1.0 / 90);
    } else if (H == 4) {
        return m == 0 ? (float)(-205.0 / 72) : m == 1 ? (float)(8.0 / 5) : m == 2 ? (float)(-1.0 / 5)
               : m == 3 ? (float)(8.0 / 315) : (float)(-1.0 / 560);
    } else if (H == 5) {
        return m == 0 ? (float)(-73766.0 / 25200) : m == 1 ? (float)(42000.0 / 25200)
               : m == 2 ? (float)(-6000.0 / 25200) : m == 3 ? (float)(1000.0 / 25200)
               : m == 4 ? (float)(-125.0 / 25200) : (float)(8.0 / 25200);
    } else {
        return m == 0 ? (float)(-2.332705821577166e+45 / 7.820582005659452e+44)
               : m == 1 ? (float)(1.3406712009703548e+45 / 7.820582005659452e+44)
               : m == 2 ? (float)(-2.0947987515168676e+44 / 7.820582005659452e+44)
               : m == 3 ? (float)(4.13787407707198e+43 / 7.820582005659452e+44)
               : m == 4 ? (float)(-6.982662505061379e+42 / 7.820582005659452e+44)
               : m == 5 ? (float)(8.12528000589218e+41 / 7.820582005659452e+44)
                        : (float)(-4.702129633040854e+40 / 7.820582005659452e+44);
    }
}

}  // namespace gbfwi
