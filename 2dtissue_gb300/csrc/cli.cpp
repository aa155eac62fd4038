// Command-line driver with the reference's flags (src/main.cpp:20-101):
//   --step-count N --particle-count N --step-time DT --mesh-path FILE.off --save-data
// plus --seed S --precision 32|64. --step-time is the time step (the reference passes it into the
// v0 slot by position, main.cpp:76-84). Prints the order-parameter series and the wall time.
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <string>

#include "tissue.hpp"

int main(int argc, char** argv) {
    int step_count = 20, particle_count = 1000, precision = 32;
    double step_time = 0.01;
    unsigned long long seed = 0;
    bool save_data = false;
    std::string mesh_path;
    for (int i = 1; i < argc; ++i) {
        std::string a = argv[i];
        auto val = [&](const char* name) -> const char* {
            if (i + 1 >= argc) {
                std::cerr << name << " needs a value\n";
                std::exit(EXIT_FAILURE);
            }
            return argv[++i];
        };
        if (a == "--step-count") step_count = std::atoi(val("--step-count"));
        else if (a == "--particle-count") particle_count = std::atoi(val("--particle-count"));
        else if (a == "--step-time") step_time = std::atof(val("--step-time"));
        else if (a == "--mesh-path") mesh_path = val("--mesh-path");
        else if (a == "--seed") seed = std::strtoull(val("--seed"), nullptr, 10);
        else if (a == "--precision") precision = std::atoi(val("--precision"));
        else if (a == "--save-data") save_data = true;
        else if (a == "--particle-innenleben" || a == "--optimized-monotile-boundary" || a == "--kafka") {
            std::cerr << a << " is not part of this implementation (ignored)\n";
        } else {
            std::cerr << "usage: " << argv[0]
                      << " [--step-count N] [--particle-count N] [--step-time DT] [--mesh-path F.off]"
                         " [--save-data] [--seed S] [--precision 32|64]\n";
            return EXIT_FAILURE;
        }
    }
    try {
        tds::Tissue2D t(save_data, false, false, mesh_path, particle_count, step_count, 0.1, false, 1, 10, 0.1,
                        0.4166666666666667, 1, 1, 0.75, step_time, 30, 1.0, 0.5, 0.0, seed, precision);
        t.start();
        auto t0 = std::chrono::steady_clock::now();
        while (!t.is_finished()) t.update();
        double s = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        for (double v : t.get_order_parameter()) std::cout << v << "\n";
        std::cout << "Time taken: " << s << " seconds\n";
    } catch (const std::exception& e) {
        std::cerr << e.what() << "\n";
        return EXIT_FAILURE;
    }
    return 0;
}
