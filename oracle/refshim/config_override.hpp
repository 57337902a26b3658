// config_override.hpp -- force-included (g++ -include) ahead of the reference sources when they
// are compiled for the oracle pin.  It defines the reference's include guard CONFIG_HPP_ first, so
// the reference's own src_cpp_kokkos_host/config.hpp is skipped and these values are used instead:
// the same names (config::, resolution_mod::) with the grid taken from -DREF_NX/NY/NZ, the domain
// from -DREF_X?MIN/MAX and one rank (ntiles = {1,1,1}).  The derived extents follow the
// reference's formulas (src_cpp_kokkos_host/config.hpp:44-69).  Test infrastructure only.
#ifndef CONFIG_HPP_
#define CONFIG_HPP_

#ifndef REF_NX
#error "REF_NX/REF_NY/REF_NZ must be given"
#endif
#ifndef REF_X1MIN
#define REF_X1MIN (-0.5)
#define REF_X1MAX (+0.5)
#define REF_X2MIN (-1.0)
#define REF_X2MAX (+1.0)
#define REF_X3MIN (-0.5)
#define REF_X3MAX (+0.5)
#endif

namespace config {
inline constexpr double time_max = 15.0e0;
inline constexpr double dtout = time_max / 100;
inline constexpr int stepmax{600000};
inline constexpr int stepsnap = stepmax / 100;
inline constexpr int ngridtotal1{REF_NX};
inline constexpr int ngridtotal2{REF_NY};
inline constexpr int ngridtotal3{REF_NZ};
inline constexpr double x1min(REF_X1MIN), x1max(REF_X1MAX);
inline constexpr double x2min(REF_X2MIN), x2max(REF_X2MAX);
inline constexpr double x3min(REF_X3MIN), x3max(REF_X3MAX);
inline constexpr int ntiles[3] = {1, 1, 1};
inline constexpr int periodic[3] = {1, 0, 1};
inline constexpr int periodicb = 1;
inline constexpr int reflection = 2;
inline constexpr int outflow = 3;
inline constexpr int boundary_xin = periodicb;
inline constexpr int boundary_xout = periodicb;
inline constexpr int boundary_yin = reflection;
inline constexpr int boundary_yout = reflection;
inline constexpr int boundary_zin = periodicb;
inline constexpr int boundary_zout = periodicb;
#ifndef REF_ASCIIOUT
#define REF_ASCIIOUT false
#endif
inline constexpr bool asciiout = REF_ASCIIOUT;
inline constexpr bool benchmarkmode = true;
};  // namespace config

namespace resolution_mod {
inline constexpr int stepmax = config::stepmax;
inline constexpr int stepsnap = config::stepsnap;
inline double time_sim = 0.0e0;
inline double time_out = 0.0e0;
inline double dt;
inline constexpr double time_max = config::time_max;
inline constexpr double dtout = config::dtout;
inline constexpr int ngrid1 = config::ngridtotal1 / config::ntiles[0];
inline constexpr int ngrid2 = config::ngridtotal2 / config::ntiles[1];
inline constexpr int ngrid3 = config::ngridtotal3 / config::ntiles[2];
inline constexpr int ngh{2};
inline constexpr int itot = ngrid1 + 2 * ngh + 1;
inline constexpr int jtot = ngrid2 + 2 * ngh + 1;
inline constexpr int ktot = ngrid3 + 2 * ngh + 1;
inline constexpr int is = ngh;
inline constexpr int js = ngh;
inline constexpr int ks = ngh;
inline constexpr int ie = is + ngrid1 - 1;
inline constexpr int je = js + ngrid2 - 1;
inline constexpr int ke = ks + ngrid3 - 1;
inline constexpr double x1min = config::x1min, x1max = config::x1max;
inline constexpr double x2min = config::x2min, x2max = config::x2max;
inline constexpr double x3min = config::x3min, x3max = config::x3max;
};  // namespace resolution_mod

#endif
