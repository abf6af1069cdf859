// Stand-in: only the traits template the functor headers specialise.
#pragma once
namespace exanb {
template <class F>
struct ComputeCellParticlesTraits {
  static inline constexpr bool RequiresBlockSynchronousCall = false;
  static inline constexpr bool CudaCompatible = false;
};
}  // namespace exanb
