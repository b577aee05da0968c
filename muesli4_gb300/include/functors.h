// functors.h -- functor concepts of the skeleton front end (drop-in for the
// reference's include/functors.h:57-410).
//
// User functors derive from Functor..Functor6 and override a MSL_USERFUNC
// operator(). The skeleton kernels are templates over the concrete functor
// type and receive the functor by value, so the call is resolved statically
// and inlined; the virtual declaration only fixes the signature.
#pragma once

#include "muesli.h"
#include "nplmatrix.h"
#include "plcube.h"
#include "plmatrix.h"

namespace msl {

template <typename T, typename R> class Functor {
   public:
    MSL_USERFUNC virtual R operator()(T value) const = 0;
    MSL_USERFUNC virtual ~Functor() {}
};
template <typename T1, typename T2, typename R> class Functor2 {
   public:
    MSL_USERFUNC virtual R operator()(T1 x, T2 y) const = 0;
    MSL_USERFUNC virtual ~Functor2() {}
};
template <typename T1, typename T2, typename T3, typename R> class Functor3 {
   public:
    MSL_USERFUNC virtual R operator()(T1 x, T2 y, T3 z) const = 0;
    MSL_USERFUNC virtual ~Functor3() {}
};
template <typename T1, typename T2, typename T3, typename T4, typename R> class Functor4 {
   public:
    MSL_USERFUNC virtual R operator()(T1 x, T2 y, T3 z, T4 v) const = 0;
    MSL_USERFUNC virtual ~Functor4() {}
};
template <typename T1, typename T2, typename T3, typename T4, typename T5, typename R> class Functor5 {
   public:
    MSL_USERFUNC virtual R operator()(T1 x, T2 y, T3 z, T4 v, T5 l) const = 0;
    MSL_USERFUNC virtual ~Functor5() {}
};
template <typename T1, typename T2, typename T3, typename T4, typename T5, typename T6, typename R> class Functor6 {
   public:
    MSL_USERFUNC virtual R operator()(T1 x, T2 y, T3 z, T4 v, T5 l, T6 m) const = 0;
    MSL_USERFUNC virtual ~Functor6() {}
};

namespace detail {
// Tile-width / shared-memory hints of the reference's stencil functor bases
// (include/detail/functor_base.h:52-182). The GB300 kernels choose their own
// tiles, so these are recorded and otherwise ignored.
class MatrixFunctorBase {
   public:
    void setTileWidth(int tw) { tile_width = tw; }
    int getTileWidth() const { return tile_width; }

   protected:
    int tile_width = DEFAULT_TILE_WIDTH;
};
}  // namespace detail

// Legacy stencil functors for DM::mapStencilMM: operator()(row, col,
// PLMatrix<T>* input, ncol, nrow) reading input->get(row, col)
// (include/functors.h:312-405).
template <typename T, typename R> class DMMapStencilFunctor : public detail::MatrixFunctorBase {
   public:
    DMMapStencilFunctor() : stencil_size(1) {}
    int getStencilSize() { return stencil_size; }
    void setStencilSize(int value) { stencil_size = value; }
    bool getSharedMemory() { return shared_memory; }
    void setSharedMemory(bool value) { shared_memory = value; }

   protected:
    int stencil_size;
    bool shared_memory = false;
};
// Base of stencil functors used with a neutral-value functor
// (DM::mapStencilMM(result, f, nvf)); the neutral-value functor type is named
// here only as in the reference, the call passes the object itself.
template <typename T, typename R, typename NeutralValueFunctor>
class DMNVFMapStencilFunctor : public DMMapStencilFunctor<T, R> {};
template <typename T, typename R, typename NeutralValueFunctor>
class MMapStencilFunctor : public DMMapStencilFunctor<T, R> {};

// Function-pointer stencil types of the current stencil API (include/functors.h:407-410).
template <typename T> using DCMapStencilFunctor = T (*)(const PLCube<T> &cs, int x, int y, int z);
template <typename T> using NPLMMapStencilFunctor = T (*)(const NPLMatrix<T> &pl, int x, int y);

}  // namespace msl
