// Prints rust_debug_f64 of every value read from stdin (one per line, as hex floats), and writes
// a small Solution with to_csv to the path given as argv[1].
#include <cstdio>
#include <cstdlib>
#include <iostream>
#include <string>

#include "degpu.hpp"

int main(int argc, char** argv) {
    std::string line;
    while (std::getline(std::cin, line)) {
        if (line.empty()) continue;
        double v = std::strtod(line.c_str(), nullptr);
        std::cout << degpu::rust_debug_f64(v) << "\n";
    }
    if (argc > 1) {
        degpu::Solution s;
        s.t = {0.0, 0.5, 1e-5};
        s.y = {{1.0, -2.5}, {1e16, 0.1}, {2.5e-300, -0.0}};
        if (!s.to_csv(argv[1])) return 1;
    }
    return 0;
}
