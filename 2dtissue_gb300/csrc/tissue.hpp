// C++ facade over the C-ABI with the reference's interface: class _2DTissue
// (src/simulation/2DTissue.h:35-60) and its Particle / System records (src/simulation/Struct.h:9-29).
// Header-only; link against lib2dtissue_gb300.so.
//
// Differences from the reference, by design:
//   * step_size is the time step; the reference CLI passes --step-time into the v0 slot
//     (main.cpp:76-84) -- the CLI here maps --step-time to step_size explicitly;
//   * errors throw std::runtime_error carrying the C-ABI message (the reference exits or throws
//     from Validation, Validation.cpp:40-72);
//   * Kafka/SQLite sinks and the particle "Innenleben" are not part of this path.
#pragma once
#include <cmath>
#include <cstddef>
#include <cstdio>
#include <filesystem>
#include <fstream>
#include <iomanip>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/tds.h"

namespace tds {

struct Particle {
    double x_UV, y_UV;
    double x_velocity_UV, y_velocity_UV;
    double alignment_UV;  // polarity angle in the chart, degrees (the reference stores int degrees)
    double compass_north_pole_UV = 0, compass_south_pole_UV = 0;  // never set by the reference either
    double x_3D, y_3D, z_3D;
    int neighbor_count;
};

struct System {
    double order_parameter;
    std::vector<Particle> particles;
};

// The C-ABI's record has the same fields in the same order: update() receives the device-packed
// records straight into System::particles.
static_assert(sizeof(Particle) == sizeof(tds_particle), "Particle and tds_particle must have one layout");
static_assert(offsetof(Particle, alignment_UV) == offsetof(tds_particle, alignment_UV), "layout");
static_assert(offsetof(Particle, x_3D) == offsetof(tds_particle, x_3D), "layout");
static_assert(offsetof(Particle, neighbor_count) == offsetof(tds_particle, neighbor_count), "layout");

class Tissue2D {
  public:
    Tissue2D(bool save_data, bool particle_innenleben, bool free_boundary, std::string mesh_path, int particle_count,
             int step_count = 1, double v0 = 0.1, bool use_kafka = false, double k = 1, double k_next = 10,
             double v0_next = 0.1, double sigma = 0.4166666666666667, double mu = 1, double r_adh = 1,
             double k_adh = 0.75, double step_size = 0.001, int map_cache_count = 30, double tau = 1.0,
             double align = 0.5, double eta = 0.0, uint64_t seed = 0, int precision = 32)
        : save_data_(save_data), n_(particle_count), step_count_(step_count) {
        (void)particle_innenleben, (void)free_boundary, (void)use_kafka, (void)k_next, (void)v0_next;
        (void)map_cache_count;
        int rc = mesh_path.empty() ? tds_mesh_ellipsoid(4, 2.0, 1.0, 1.0, &mesh_)
                                   : tds_mesh_load_off(mesh_path.c_str(), &mesh_);
        if (rc) throw std::runtime_error(std::string("mesh: ") + tds_mesh_last_error());
        tds_params p{};
        p.radius = sigma;
        p.k_rep = k;
        p.k_adh = k_adh;
        p.r_max = r_adh;
        p.v0 = v0;
        p.mu = mu;
        p.tau = tau;
        p.align = align;
        p.eta = eta;
        p.dt = step_size;
        p.force_mode = 0;
        rc = tds_create(mesh_, &p, particle_count, seed, precision, &sim_);
        if (rc) {
            tds_mesh_destroy(mesh_);
            throw std::runtime_error("tds_create failed (code " + std::to_string(rc) + ")");
        }
    }
    Tissue2D(const Tissue2D&) = delete;
    Tissue2D& operator=(const Tissue2D&) = delete;
    ~Tissue2D() {
        tds_destroy(sim_);
        tds_mesh_destroy(mesh_);
    }

    void start() { check(tds_start(sim_)); }

    System update() {
        check(tds_step(sim_, 1, nullptr));
        ++current_step_;
        System sys;
        int ns = 0;
        std::vector<double> phi(current_step_);
        check(tds_get_order_parameter(sim_, phi.data(), nullptr, (int)phi.size(), &ns));
        sys.order_parameter = ns > 0 ? phi[ns - 1] : 0.0;
        sys.particles.resize(n_);
        check(tds_get_particles(sim_, reinterpret_cast<tds_particle*>(sys.particles.data())));
        if (save_data_) save_our_data(sys.particles);
        return sys;
    }

    bool is_finished() const { return current_step_ >= step_count_; }

    std::vector<double> get_order_parameter() {
        std::vector<double> phi(step_count_, 0.0);
        int ns = 0;
        check(tds_get_order_parameter(sim_, phi.data(), nullptr, step_count_, &ns));
        return phi;
    }

    tds_sim* handle() { return sim_; }

  private:
    void check(int rc) {
        if (rc) throw std::runtime_error(std::string("tds: ") + tds_last_error(sim_));
    }
    // CSV layout of save_matrix_to_csv (IO.h:40-69): 15 significant digits, one row per particle,
    // files r_data_<step>.csv, r_data_3D_<step>.csv, particles_color_<step>.csv in ./data, opened
    // in append mode as the reference opens them (IO.h:44), so that a run into a data/ directory
    // that already holds files of an earlier run adds its rows after theirs.
    void save_our_data(const std::vector<Particle>& ps) {
        std::filesystem::create_directories("data");
        const std::string k = std::to_string(current_step_);
        std::ofstream uv("data/r_data_" + k + ".csv", std::ios::app), r3("data/r_data_3D_" + k + ".csv", std::ios::app);
        std::ofstream nb("data/particles_color_" + k + ".csv", std::ios::app);
        uv << std::setprecision(15);
        r3 << std::setprecision(15);
        for (const Particle& q : ps) {
            uv << q.x_UV << "," << q.y_UV << "\n";
            r3 << q.x_3D << "," << q.y_3D << "," << q.z_3D << "\n";
            nb << q.neighbor_count << "\n";
        }
    }

    bool save_data_;
    int n_, step_count_, current_step_ = 0;
    tds_mesh* mesh_ = nullptr;
    tds_sim* sim_ = nullptr;
};

}  // namespace tds
