// illum_gb300.hpp — header-only C++ front-end over illum_gb300.h with the
// names, argument meaning and error behaviour (exceptions) of sampotter/illum's
// C++ API, so a caller of the reference's library can switch by changing the
// include and the link line:
//
//   illum_gb300::illum_context      ~ illum_context     (src/cpp/illum.hpp:6-48)
//   illum_gb300::thermal_model      ~ thermal_model     (src/cpp/thermal.hpp:7-127)
//   illum_gb300::fib_spiral         ~ fib_spiral        (src/cpp/illum.cpp:468-483)
//   illum_gb300::conductionQ / T    ~ conductionQ / T   (src/cpp/conduction.hpp:4-28)
//
// Armadillo types are replaced by std::vector (column-major where the
// reference uses arma::mat) and a plain CSR struct for arma::sp_mat; the
// reference's boost::variant arguments become overloads.
#ifndef ILLUM_GB300_HPP
#define ILLUM_GB300_HPP

#include <stdexcept>
#include <string>
#include <vector>

#include "illum_gb300.h"

namespace illum_gb300 {

inline void check(int rc) {
  if (rc != ILG_OK) throw std::runtime_error(std::string("illum_gb300: ") + ilg_last_error());
}

// Form-factor matrix, CSR by receiver row i (the reference's sp_mat F with
// F(i, j) = albedo_i * F_ij).
struct csr_matrix {
  int n = 0;
  std::vector<int64_t> rowptr;
  std::vector<int32_t> col;
  std::vector<double> val;
  size_t n_nonzero() const { return val.size(); }
};

// xy: n x 2 column-major.
inline void fib_spiral(std::vector<double>& xy, int n) {
  xy.assign(2 * (size_t)n, 0.0);
  ilg_fib_spiral(xy.data(), n);
}

class illum_context {
 public:
  // verts: nv x 3 row-major float; faces: nt x 3 vertex indices (the OBJ's
  // triangles); normals: optional per-face normals (oriented as the
  // reference orients them, src/cpp/obj_util.cpp:70-88).
  illum_context(const std::vector<float>& verts, const std::vector<int32_t>& faces,
                const std::vector<float>* normals = nullptr)
      : num_faces((int)(faces.size() / 3)) {
    check(ilg_ctx_create(verts.data(), (int)(verts.size() / 3), faces.data(), num_faces,
                         normals ? normals->data() : nullptr, &h_));
  }
  illum_context(const illum_context&) = delete;
  illum_context& operator=(const illum_context&) = delete;
  ~illum_context() { ilg_ctx_destroy(h_); }

  int get_num_faces() const { return num_faces; }

  csr_matrix compute_F(double albedo, double offset = 1e-5) { return compute_F_(nullptr, albedo, offset); }
  csr_matrix compute_F(const std::vector<double>& albedo, double offset = 1e-5) {
    return compute_F_(albedo.data(), 1.0, offset);
  }

  // A separate mesh the horizon rays are traced against (the reference's
  // set_horizon_obj_file, illum.hpp:36-37; here the loaded triangles:
  // vertices nv x 3 row-major float, faces nt x 3).
  void set_horizon_mesh(const std::vector<float>& verts, const std::vector<int32_t>& faces) {
    hverts_ = verts;
    hfaces_ = faces;
  }
  void make_horizons(int nphi = 361, double theta_eps = 1e-3, double offset = 1e-5) {
    if (hfaces_.empty())
      check(ilg_make_horizons(h_, nphi, theta_eps, offset));
    else
      check(ilg_make_horizons_mesh(h_, hverts_.data(), (int)(hverts_.size() / 3), hfaces_.data(),
                                   (int)(hfaces_.size() / 3), nphi, theta_eps, offset));
    nphi_ = nphi;
  }
  // nphi x N column-major, as the reference's arma::mat horizons.
  std::vector<double> horizons() const {
    std::vector<double> h((size_t)nphi_ * num_faces);
    check(ilg_get_horizons(h_, h.data()));
    return h;
  }
  void load_horizons(const std::vector<double>& h, int nphi) {
    check(ilg_set_horizons(h_, nphi, h.data()));
    nphi_ = nphi;
  }

  // sun_position: 3 values (km); disk_xy: n x 2 column-major.
  std::vector<double> get_direct_radiosity(const std::vector<double>& sun_position, const std::vector<double>& disk_xy) {
    std::vector<double> out(num_faces);
    check(ilg_direct_radiosity(h_, sun_position.data(), disk_xy.data(), (int)(disk_xy.size() / 2), out.data()));
    return out;
  }

  // (I - F) x = E to ||(I - F) x - E||_2 <= tol: the system the reference
  // solves with arma_util::forward_solve and Gauss-Seidel sweeps.
  std::vector<double> radiosity(const std::vector<double>& E, double tol = 1e-10, int max_sweeps = 200) {
    std::vector<double> x(num_faces);
    check(ilg_radiosity_solve(h_, E.data(), tol, max_sweeps, x.data(), nullptr, nullptr));
    return x;
  }

  // The reference's own solve (illum_cli.cpp:425-433): forward solve plus
  // gs_steps natural-order Gauss-Seidel sweeps.
  std::vector<double> radiosity_gs(const std::vector<double>& E, int gs_steps = 1, double* res = nullptr) {
    std::vector<double> x(num_faces);
    check(ilg_radiosity_solve_gs(h_, E.data(), gs_steps, x.data(), res));
    return x;
  }

  ilg_ctx* handle() { return h_; }
  const int num_faces;

 private:
  csr_matrix compute_F_(const double* alb, double scalar, double offset) {
    int64_t nnz = 0, rays = 0;
    check(ilg_compute_F(h_, alb, scalar, offset, &nnz, &rays));
    csr_matrix F;
    F.n = num_faces;
    F.rowptr.resize((size_t)num_faces + 1);
    F.col.resize((size_t)nnz);
    F.val.resize((size_t)nnz);
    check(ilg_get_F(h_, F.rowptr.data(), F.col.data(), F.val.data()));
    return F;
  }
  ilg_ctx* h_ = nullptr;
  int nphi_ = 0;
  std::vector<float> hverts_;
  std::vector<int32_t> hfaces_;
};

class thermal_model {
 public:
  // Same arguments as the reference's constructor (thermal.hpp:17-59);
  // emissivity defaults to the reference's hard-coded 0.999 (thermal.hpp:77).
  thermal_model(illum_context& ctx, const std::vector<double>& depths, double thermal_inertia, double rhoc,
                double init_temp, double emissivity = 0.999, int bc_mode = ILG_BC_LINEARISED,
                int precision = ILG_PREC_FP64)
      : ctx_(ctx), nz((int)depths.size()) {
    std::vector<double> ti(nz, thermal_inertia), rc(nz, rhoc);
    check(ilg_thermal_init(ctx.handle(), nz, depths.data(), ti.data(), rc.data(), init_temp, nullptr, emissivity, 0.0,
                           bc_mode, precision));
  }
  void step(double dt, const std::vector<double>& Q) {
    check(ilg_thermal_step(ctx_.handle(), dt, Q.data()));
    t += dt;
  }
  // (nz+1) x N column-major, row 0 = surface temperature.
  std::vector<double> T() const {
    std::vector<double> out((size_t)(nz + 1) * ctx_.num_faces);
    check(ilg_thermal_get(ctx_.handle(), out.data(), nullptr, nullptr));
    return out;
  }
  std::vector<double> get_radiosity() const {
    std::vector<double> F(ctx_.num_faces);
    check(ilg_thermal_get(ctx_.handle(), nullptr, F.data(), nullptr));
    for (double& x : F) x = -x;
    return F;
  }

 private:
  illum_context& ctx_;

 public:
  const int nz;
  double t = 0.0;
};

inline void conductionQ(int nz, const double* z, double dt, double Qn, double Qnp1, double* T, const double* ti,
                        const double* rhoc, double emiss, double* Tsurf, double Fgeotherm, double* Fsurf) {
  conductionq_(&nz, z, &dt, &Qn, &Qnp1, T, ti, rhoc, &emiss, Tsurf, &Fgeotherm, Fsurf);
}

inline void conductionT(int nz, const double* z, double dt, double* T, double Tsurf, double Tsurfp1, const double* ti,
                        const double* rhoc, double Fgeotherm, double* Fsurf) {
  conductiont_(&nz, z, &dt, T, &Tsurf, &Tsurfp1, ti, rhoc, &Fgeotherm, Fsurf);
}

}  // namespace illum_gb300

#endif  // ILLUM_GB300_HPP
