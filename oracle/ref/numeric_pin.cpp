// Runs the reference's own approxExactlyDivisible (include/flamegpu/detail/numeric.h:24-31,
// compiled from the reference tree) over a grid of (width, radius) pairs and prints
// JSON lines {"x":..,"y":..,"r":0|1}. The oracle's restatement is checked against it.
#include <cstdio>
#include <cstring>
#include "flamegpu/detail/numeric.h"

int main() {
    const float widths[] = {1.0f, 5.0f, 11.0f, 30.0f, 50.1f, 64.0f, 70.0f, 0.3f, 1000.0f, 4096.0f, 256.0f, 7.5f, 9.9f, 100.0f};
    const float radii[] = {0.05f, 0.1f, 0.5f, 1.0f, 2.0f, 3.0f, 3.5f, 4.0f, 10.0f, 0.3f, 1.5f, 2.5f, 0.7f, 0.01f};
    std::printf("[\n");
    bool first = true;
    for (float w : widths)
        for (float r : radii) {
            unsigned ux, ur;
            std::memcpy(&ux, &w, 4);
            std::memcpy(&ur, &r, 4);
            std::printf("%s{\"x_bits\": %u, \"y_bits\": %u, \"r\": %d}", first ? "" : ",\n", ux, ur,
                        flamegpu::detail::numeric::approxExactlyDivisible<float>(w, r) ? 1 : 0);
            first = false;
        }
    std::printf("\n]\n");
    return 0;
}
