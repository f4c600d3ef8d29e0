// FleCSI-side wrapper library, ocean app: every task of
// apps/ocean/tasks/solve.hh with the reference's exact signature, built in
// place of apps/ocean/tasks/solve.cc.  The FCT and del2 tasks (solve.cc:40-399)
// call libmpaso's per-task entries; the copy / zero tasks stay on the host.
// The FCT statics the signatures pass (maxLevelCell, advCoef, ...) were given
// to the device context once (make_mesh_context with FctStatics).
#include "apps/ocean/state.hh"
#include "apps/ocean/tasks/solve.hh"
#include "mpaso_flecsi.hh"

namespace mpas { namespace ocean { namespace task {

using namespace flecsi;
using mpaso_flecsi::context;
using mpaso_flecsi::ok;
using mpaso_flecsi::raw;

namespace {
constexpr int32_t kL = (int32_t)nVertLevels, kT = (int32_t)maxTracers;
}

void copy_tracers(mesh::accessor<ro, ro> m, acc<vltracer, ro, ro> tracers, acc<vltracer, wo, na> tracersNew,
                  acc<vltracer, wo, na> tracersPrev) {
  for (auto c : m.cells()) tracersNew(c) = tracers(c), tracersPrev(c) = tracers(c);
}

void reinitialize_tracer_tendencies(mesh::accessor<ro, ro> m, acc<vltracer, wo, na> tend) {
  for (auto c : m.cells()) tend(c) = vltracer{};
}

void calc_normal_thickness_flux(mesh::accessor<ro, ro>, acc<vltensor<double>, ro, ro> layerThicknessEdge,
                                acc<vltensor<double>, ro, ro> normalVelocity,
                                acc<vltensor<double>, wo, na> normalThicknessFlux) {
  ok(mpaso_oc_calc_normal_thickness_flux(context(), kL, raw(layerThicknessEdge), raw(normalVelocity),
                                         raw(normalThicknessFlux), nullptr));
}

void calc_provisional_layer_thicknesses(mesh::accessor<ro, ro>, acc<int, ro, ro>, acc<double, ro, ro>,
                                        acc<double, ro, ro>, acc<metensor<double>, ro, ro>,
                                        acc<vltensor<double>, ro, ro> layerThickness,
                                        acc<vltensor<double>, ro, ro> normalThicknessFlux,
                                        acc<vltensor<double>, ro, ro>, acc<vltensor<double>, wo, na> hProv,
                                        acc<vltensor<double>, wo, na> hProvInv,
                                        acc<vltensor<double>, wo, na> hNewInv, double dt) {
  ok(mpaso_oc_calc_provisional_layer_thicknesses(context(), kL, raw(layerThickness), raw(normalThicknessFlux),
                                                 raw(hProv), raw(hProvInv), raw(hNewInv), dt, nullptr));
}

void calc_horiz_tracer_advection_flux_mono_low_order(mesh::accessor<ro, ro>, acc<double, ro, ro>,
                                                     acc<vltensor<double>, ro, ro> normalThicknessFlux,
                                                     acc<vltracer, ro, ro> tracers,
                                                     acc<vltracer, wo, na> lowOrderFlux) {
  ok(mpaso_oc_calc_horiz_tracer_advection_flux_mono_low_order(context(), kL, kT, raw(normalThicknessFlux),
                                                              raw(tracers), raw(lowOrderFlux), nullptr));
}

void calc_horiz_tracer_advection_flux_mono_high_order(
    mesh::accessor<ro, ro>, acc<vltensor<int>, ro, ro>, acc<double, ro, ro>,
    acc<vltensor<double>, ro, ro> normalThicknessFlux, acc<me2tensor<double>, ro, ro>, acc<me2tensor<double>, ro, ro>,
    acc<int, ro, ro>, acc<int, ro, ro>, acc<me2tensor<int>, ro, ro>, acc<vltracer, ro, ro> tracers,
    acc<vltracer, wo, na> highOrderFlux) {
  ok(mpaso_oc_calc_horiz_tracer_advection_flux_mono_high_order(context(), kL, kT, raw(normalThicknessFlux),
                                                               raw(tracers), raw(highOrderFlux), nullptr));
}

void correct_and_rescale_high_order_mono_horiz_flux(
    mesh::accessor<ro, ro>, acc<metensor<double>, ro, ro>, acc<vltensor<double>, ro, ro> hProvInv,
    acc<vltensor<double>, ro, ro> layerThickness, acc<vltensor<double>, ro, ro> normalThicknessFlux,
    acc<double, ro, ro>, acc<double, ro, ro>, acc<vltensor<int>, ro, ro>, acc<int, ro, ro>, acc<int, ro, ro>,
    acc<vltracer, ro, ro> lowOrderFlux, acc<vltracer, ro, ro> tracers, acc<vltracer, rw, ro> highOrderFlux,
    acc<vltracer, wo, na> flxIn, acc<vltracer, wo, na> flxOut, acc<vltracer, wo, na> tend,
    acc<vltracer, wo, na> tracerMax, acc<vltracer, wo, na> tracerMin, double dt) {
  ok(mpaso_oc_correct_and_rescale_high_order_mono_horiz_flux(
      context(), kL, kT, raw(hProvInv), raw(layerThickness), raw(normalThicknessFlux), raw(lowOrderFlux),
      raw(tracers), raw(highOrderFlux), raw(flxIn), raw(flxOut), raw(tend), raw(tracerMax), raw(tracerMin), dt,
      nullptr));
}

void accumulate_horiz_tracer_advection_tend_mono_FCT(
    mesh::accessor<ro, ro>, acc<metensor<double>, ro, ro>, acc<vltensor<double>, ro, ro> hProvInv,
    acc<vltensor<double>, ro, ro> layerThickness, acc<double, ro, ro>, acc<int, ro, ro>, acc<int, ro, ro>,
    acc<vltracer, ro, ro> highOrderFlux, acc<vltracer, ro, ro> tracers, acc<vltracer, wo, na> tracersProv,
    acc<vltracer, rw, ro> tend, double dt) {
  ok(mpaso_oc_accumulate_horiz_tracer_advection_tend_mono_FCT(context(), kL, kT, raw(hProvInv), raw(layerThickness),
                                                              raw(highOrderFlux), raw(tracers), raw(tracersProv),
                                                              raw(tend), dt, nullptr));
}

void tracer_hmix_del2_tend(mesh::accessor<ro, ro>, acc<double, ro, ro>, acc<double, ro, ro>, acc<double, ro, ro>,
                           acc<double, ro, ro>, acc<int, ro, ro>, acc<metensor<double>, ro, ro>,
                           acc<vltensor<double>, ro, ro> layerThicknessEdge, acc<vltracer, ro, ro> tracers,
                           acc<vltracer, rw, ro> tend, double coef) {
  ok(mpaso_oc_tracer_hmix_del2_tend(context(), kL, kT, raw(layerThicknessEdge), raw(tracers), raw(tend), coef,
                                    nullptr));
}

void step_tracers_forward(mesh::accessor<ro, ro>, acc<vltracer, ro, ro> tend, acc<vltracer, ro, ro> tracers,
                          acc<vltracer, rw, ro> tracersNew, acc<vltracer, wo, na> tracersPrev, double rk_weight,
                          double rk_subweight) {
  ok(mpaso_oc_step_tracers_forward(context(), kL, kT, raw(tend), raw(tracers), raw(tracersNew), raw(tracersPrev),
                                   rk_weight, rk_subweight, nullptr));
}

void update_tracers(mesh::accessor<ro, ro> m, acc<vltracer, ro, ro> tracersNew, acc<vltracer, wo, na> tracers) {
  for (auto c : m.cells()) tracers(c) = tracersNew(c);
}

}}}  // namespace mpas::ocean::task
