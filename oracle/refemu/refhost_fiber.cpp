/*
 * refhost_fiber.cpp -- the reference's fibrin code (fiber.cpp, included from
 * the reference tree at build time, with network.cpp linked beside it) on
 * the CPU, exposing its worm-like-chain law (fiber.cpp:710-733, a static
 * function there) to pin the oracle's restatement of it.
 * ORACLE TEST INFRASTRUCTURE ONLY: built by oracle/refemu/build_refemu.sh into
 * oracle/_ref/ where the reference tree is present; never shipped or linked by
 * the product.
 */
#include "fiber.cpp"

extern "C" double refhost_wlc(double ini_l, double cur_l, double modulus, double mass) {
  return wormlike_chain_force(ini_l, cur_l, modulus, mass);
}
