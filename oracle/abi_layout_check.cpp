// abi_layout_check.cpp -- compile-time proof that libbhk's C structs are layout-identical to the
// reference's kerr:: structs they stand in for (src/kerr.h:81-99, 143-145), so a maintainer may
// pass kerr::Constants / State / Derivatives / Frame to the bhk_* mirrors by pointer cast.
//
// TEST INFRASTRUCTURE ONLY: compiled (-fsyntax-only) by `make -C oracle ref` where the reference
// headers exist; it produces no object and nothing links it.
#include <cstddef>
#include <type_traits>

#include "kerr.h"

#include "../include/bhk.h"

#define SAME_FIELD(A, B, fa, fb) static_assert(offsetof(A, fa) == offsetof(B, fb), #A "." #fa " offset")

static_assert(sizeof(bhk_constants) == sizeof(kerr::Constants), "constants size");
SAME_FIELD(bhk_constants, kerr::Constants, E, E);
SAME_FIELD(bhk_constants, kerr::Constants, L, L);
SAME_FIELD(bhk_constants, kerr::Constants, Q, Q);
SAME_FIELD(bhk_constants, kerr::Constants, mu, mu);

static_assert(sizeof(bhk_state) == sizeof(kerr::State), "state size");
SAME_FIELD(bhk_state, kerr::State, t, t);
SAME_FIELD(bhk_state, kerr::State, r, r);
SAME_FIELD(bhk_state, kerr::State, theta, theta);
SAME_FIELD(bhk_state, kerr::State, phi, phi);
SAME_FIELD(bhk_state, kerr::State, vr, vr);
SAME_FIELD(bhk_state, kerr::State, vtheta, vtheta);

static_assert(sizeof(bhk_derivatives_t) == sizeof(kerr::Derivatives), "derivatives size");
SAME_FIELD(bhk_derivatives_t, kerr::Derivatives, dt, dt);
SAME_FIELD(bhk_derivatives_t, kerr::Derivatives, dr, dr);
SAME_FIELD(bhk_derivatives_t, kerr::Derivatives, dtheta, dtheta);
SAME_FIELD(bhk_derivatives_t, kerr::Derivatives, dphi, dphi);
SAME_FIELD(bhk_derivatives_t, kerr::Derivatives, dvr, dvr);
SAME_FIELD(bhk_derivatives_t, kerr::Derivatives, dvtheta, dvtheta);

// kerr::Frame is four std::array<double, 4> (e[k] the k-th tetrad vector), bhk_frame double e[4][4].
static_assert(sizeof(kerr::Vec4) == 4 * sizeof(double), "Vec4 is four packed doubles");
static_assert(sizeof(bhk_frame) == sizeof(kerr::Frame), "frame size");
SAME_FIELD(bhk_frame, kerr::Frame, e, e);

static_assert(std::is_standard_layout<kerr::Constants>::value && std::is_standard_layout<kerr::State>::value &&
                  std::is_standard_layout<kerr::Derivatives>::value && std::is_standard_layout<kerr::Frame>::value,
              "the reference structs are plain data");
