// Count of kernel launches made by this library (reported by kgb_launch_count).
#pragma once

namespace kgb {
void count_launch(int n = 1);
}  // namespace kgb
