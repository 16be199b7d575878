! emdee.f03 -- Fortran interface to the GB300 EmDee library (libemdee.so).
!
! Same types and entry points as the reference's Fortran header
! (src/emdee_header.f03:21-262 and the generated model factories), so host
! programs that include it compile unchanged.  Layout pinned in include/emdee.h.

module EmDee

use iso_c_binding

implicit none

type, bind(C) :: tOpts
  logical(c_bool) :: Translate
  logical(c_bool) :: Rotate
  integer(c_int)  :: RotationMode
  logical(c_bool) :: AutoForceCompute
  logical(c_bool) :: AutoBodyUpdate
  logical(c_bool) :: Compute
end type tOpts

type, bind(C) :: tEnergy
  real(c_double)  :: Potential
  real(c_double)  :: Dispersion
  real(c_double)  :: Coulomb
  real(c_double)  :: Bond
  real(c_double)  :: Angle
  real(c_double)  :: Dihedral
  real(c_double)  :: ShadowPotential
  logical(c_bool) :: UpToDate
end type tEnergy

type, bind(C) :: tKinetic
  real(c_double)  :: Total
  real(c_double)  :: TransPart(3)
  real(c_double)  :: Rotational
  real(c_double)  :: RotPart(3)
  real(c_double)  :: ShadowKinetic
  real(c_double)  :: ShadowRotational
  logical(c_bool) :: UpToDate
end type tKinetic

type, bind(C) :: tVirial
  real(c_double) :: Total
  real(c_double) :: Body
end type tVirial

type, bind(C) :: tTime
  real(c_double) :: Pair
  real(c_double) :: Motion
  real(c_double) :: Neighbor
  real(c_double) :: Total
end type tTime

type, bind(C) :: tEmDee
  integer(c_int)  :: Builds
  type(tTime)     :: Time
  type(tEnergy)   :: Energy
  type(tKinetic)  :: Kinetic
  type(tVirial)   :: Virial
  integer(c_int)  :: DoF
  integer(c_int)  :: RotDoF
  type(c_ptr)     :: Data
  type(tOpts)     :: Options
end type tEmDee

interface

  function EmDee_system( threads, layers, rc, skin, N, types, masses, bodies ) bind(C,name="EmDee_system")
    import
    integer(c_int), value :: threads
    integer(c_int), value :: layers
    real(c_double), value :: rc
    real(c_double), value :: skin
    integer(c_int), value :: N
    type(c_ptr), value :: types
    type(c_ptr), value :: masses
    type(c_ptr), value :: bodies
    tEmDee :: EmDee_system
  end function EmDee_system

  function EmDee_memory_address( md, option ) bind(C,name="EmDee_memory_address")
    import
    type(tEmDee), value :: md
    character(c_char), intent(in) :: option(*)
    type(c_ptr) :: EmDee_memory_address
  end function EmDee_memory_address

  subroutine EmDee_share_phase_space( mdkeep, mdlose ) bind(C,name="EmDee_share_phase_space")
    import
    type(tEmDee), value :: mdkeep
    type(tEmDee), intent(inout) :: mdlose
  end subroutine EmDee_share_phase_space

  subroutine EmDee_layer_based_parameters( md, InternalRc, Apply, Bonded ) bind(C,name="EmDee_layer_based_parameters")
    import
    type(tEmDee), value :: md
    real(c_double), value :: InternalRc
    integer(c_int), intent(in) :: Apply(*)
    integer(c_int), intent(in) :: Bonded(*)
  end subroutine EmDee_layer_based_parameters

  subroutine EmDee_set_pair_model( md, itype, jtype, model, kCoul ) bind(C,name="EmDee_set_pair_model")
    import
    type(tEmDee), value :: md
    integer(c_int), value :: itype
    integer(c_int), value :: jtype
    type(c_ptr), value :: model
    real(c_double), value :: kCoul
  end subroutine EmDee_set_pair_model

  subroutine EmDee_set_pair_multimodel( md, itype, jtype, model, kCoul ) bind(C,name="EmDee_set_pair_multimodel")
    import
    type(tEmDee), value :: md
    integer(c_int), value :: itype
    integer(c_int), value :: jtype
    type(c_ptr), intent(in) :: model(*)
    real(c_double), intent(in) :: kCoul(*)
  end subroutine EmDee_set_pair_multimodel

  subroutine EmDee_set_kspace_model( md, model ) bind(C,name="EmDee_set_kspace_model")
    import
    type(tEmDee), value :: md
    type(c_ptr), value :: model
  end subroutine EmDee_set_kspace_model

  subroutine EmDee_set_coul_model( md, model ) bind(C,name="EmDee_set_coul_model")
    import
    type(tEmDee), value :: md
    type(c_ptr), value :: model
  end subroutine EmDee_set_coul_model

  subroutine EmDee_set_coul_multimodel( md, model ) bind(C,name="EmDee_set_coul_multimodel")
    import
    type(tEmDee), value :: md
    type(c_ptr), intent(in) :: model(*)
  end subroutine EmDee_set_coul_multimodel

  subroutine EmDee_ignore_pair( md, i, j ) bind(C,name="EmDee_ignore_pair")
    import
    type(tEmDee), value :: md
    integer(c_int), value :: i
    integer(c_int), value :: j
  end subroutine EmDee_ignore_pair

  subroutine EmDee_add_bond( md, i, j, model ) bind(C,name="EmDee_add_bond")
    import
    type(tEmDee), value :: md
    integer(c_int), value :: i
    integer(c_int), value :: j
    type(c_ptr), value :: model
  end subroutine EmDee_add_bond

  subroutine EmDee_add_angle( md, i, j, k, model ) bind(C,name="EmDee_add_angle")
    import
    type(tEmDee), value :: md
    integer(c_int), value :: i
    integer(c_int), value :: j
    integer(c_int), value :: k
    type(c_ptr), value :: model
  end subroutine EmDee_add_angle

  subroutine EmDee_add_dihedral( md, i, j, k, l, model ) bind(C,name="EmDee_add_dihedral")
    import
    type(tEmDee), value :: md
    integer(c_int), value :: i
    integer(c_int), value :: j
    integer(c_int), value :: k
    integer(c_int), value :: l
    type(c_ptr), value :: model
  end subroutine EmDee_add_dihedral

  subroutine EmDee_download( md, option, address ) bind(C,name="EmDee_download")
    import
    type(tEmDee), value :: md
    character(c_char), intent(in) :: option(*)
    type(c_ptr), value :: address
  end subroutine EmDee_download

  subroutine EmDee_upload( md, option, address ) bind(C,name="EmDee_upload")
    import
    type(tEmDee), intent(inout) :: md
    character(c_char), intent(in) :: option(*)
    type(c_ptr), value :: address
  end subroutine EmDee_upload

  subroutine EmDee_switch_model_layer( md, layer ) bind(C,name="EmDee_switch_model_layer")
    import
    type(tEmDee), intent(inout) :: md
    integer(c_int), value :: layer
  end subroutine EmDee_switch_model_layer

  subroutine EmDee_random_momenta( md, kT, adjust, seed ) bind(C,name="EmDee_random_momenta")
    import
    type(tEmDee), intent(inout) :: md
    real(c_double), value :: kT
    logical(c_bool), value :: adjust
    integer(c_int), value :: seed
  end subroutine EmDee_random_momenta

  subroutine EmDee_boost( md, lambda, alpha, dt ) bind(C,name="EmDee_boost")
    import
    type(tEmDee), intent(inout) :: md
    real(c_double), value :: lambda
    real(c_double), value :: alpha
    real(c_double), value :: dt
  end subroutine EmDee_boost

  subroutine EmDee_displace( md, lambda, alpha, dt ) bind(C,name="EmDee_displace")
    import
    type(tEmDee), intent(inout) :: md
    real(c_double), value :: lambda
    real(c_double), value :: alpha
    real(c_double), value :: dt
  end subroutine EmDee_displace

  subroutine EmDee_move( md, lambda, alpha, dt ) bind(C,name="EmDee_move")
    import
    type(tEmDee), intent(inout) :: md
    real(c_double), value :: lambda
    real(c_double), value :: alpha
    real(c_double), value :: dt
  end subroutine EmDee_move

  subroutine EmDee_verlet_step( md, dt ) bind(C,name="EmDee_verlet_step")
    import
    type(tEmDee), intent(inout) :: md
    real(c_double), value :: dt
  end subroutine EmDee_verlet_step

  subroutine EmDee_compute_forces( md ) bind(C,name="EmDee_compute_forces")
    import
    type(tEmDee), intent(inout) :: md
  end subroutine EmDee_compute_forces

  subroutine EmDee_rdf( md, bins, Rc, pairs, itype, jtype, g ) bind(C,name="EmDee_rdf")
    import
    type(tEmDee), value :: md
    integer(c_int), value :: bins
    real(c_double), value :: Rc
    integer(c_int), value :: pairs
    integer(c_int), intent(in) :: itype(*)
    integer(c_int), intent(in) :: jtype(*)
    real(c_double), intent(out) :: g(*)
  end subroutine EmDee_rdf

  subroutine EmDee_set_precision( md, mode ) bind(C,name="EmDee_set_precision")
    import
    type(tEmDee), value :: md
    integer(c_int), value :: mode
  end subroutine EmDee_set_precision

  subroutine EmDee_set_outer_skin( md, delta ) bind(C,name="EmDee_set_outer_skin")
    import
    type(tEmDee), value :: md
    real(c_double), value :: delta
  end subroutine EmDee_set_outer_skin

  integer(c_long) function EmDee_outer_builds( md ) bind(C,name="EmDee_outer_builds")
    import
    type(tEmDee), value :: md
  end function EmDee_outer_builds

  integer(c_int) function EmDee_tile_edge( md ) bind(C,name="EmDee_tile_edge")
    import
    type(tEmDee), value :: md
  end function EmDee_tile_edge

  integer(c_int) function EmDee_tile_threads( md, kernel ) bind(C,name="EmDee_tile_threads")
    import
    type(tEmDee), value :: md
    integer(c_int), value :: kernel
  end function EmDee_tile_threads

  subroutine EmDee_destroy( md ) bind(C,name="EmDee_destroy")
    import
    type(tEmDee), intent(inout) :: md
  end subroutine EmDee_destroy

  type(c_ptr) function EmDee_shifted( model ) bind(C,name="EmDee_shifted")
    import
    type(c_ptr), value :: model
  end function EmDee_shifted

  type(c_ptr) function EmDee_shifted_force( model ) bind(C,name="EmDee_shifted_force")
    import
    type(c_ptr), value :: model
  end function EmDee_shifted_force

  type(c_ptr) function EmDee_smoothed( model, skin ) bind(C,name="EmDee_smoothed")
    import
    type(c_ptr), value :: model
    real(c_double), value :: skin
  end function EmDee_smoothed

  type(c_ptr) function EmDee_shifted_smoothed( model, skin ) bind(C,name="EmDee_shifted_smoothed")
    import
    type(c_ptr), value :: model
    real(c_double), value :: skin
  end function EmDee_shifted_smoothed

  type(c_ptr) function EmDee_square_smoothed( model, skin ) bind(C,name="EmDee_square_smoothed")
    import
    type(c_ptr), value :: model
    real(c_double), value :: skin
  end function EmDee_square_smoothed

  type(c_ptr) function EmDee_shifted_square_smoothed( model, skin ) bind(C,name="EmDee_shifted_square_smoothed")
    import
    type(c_ptr), value :: model
    real(c_double), value :: skin
  end function EmDee_shifted_square_smoothed

  type(c_ptr) function EmDee_pair_none(  ) bind(C,name="EmDee_pair_none")
    import
  end function EmDee_pair_none

  type(c_ptr) function EmDee_coul_none(  ) bind(C,name="EmDee_coul_none")
    import
  end function EmDee_coul_none

  type(c_ptr) function EmDee_bond_none(  ) bind(C,name="EmDee_bond_none")
    import
  end function EmDee_bond_none

  type(c_ptr) function EmDee_angle_none(  ) bind(C,name="EmDee_angle_none")
    import
  end function EmDee_angle_none

  type(c_ptr) function EmDee_dihedral_none(  ) bind(C,name="EmDee_dihedral_none")
    import
  end function EmDee_dihedral_none

  type(c_ptr) function EmDee_pair_lj_cut( epsilon, sigma ) bind(C,name="EmDee_pair_lj_cut")
    import
    real(c_double), value :: epsilon
    real(c_double), value :: sigma
  end function EmDee_pair_lj_cut

  type(c_ptr) function EmDee_pair_softcore_cut( epsilon, sigma, lambda ) bind(C,name="EmDee_pair_softcore_cut")
    import
    real(c_double), value :: epsilon
    real(c_double), value :: sigma
    real(c_double), value :: lambda
  end function EmDee_pair_softcore_cut

  type(c_ptr) function EmDee_coul_cut(  ) bind(C,name="EmDee_coul_cut")
    import
  end function EmDee_coul_cut

  type(c_ptr) function EmDee_coul_sf(  ) bind(C,name="EmDee_coul_sf")
    import
  end function EmDee_coul_sf

  type(c_ptr) function EmDee_coul_damped( damp ) bind(C,name="EmDee_coul_damped")
    import
    real(c_double), value :: damp
  end function EmDee_coul_damped

  type(c_ptr) function EmDee_coul_damped_smoothed( damp, skinWidth ) bind(C,name="EmDee_coul_damped_smoothed")
    import
    real(c_double), value :: damp
    real(c_double), value :: skinWidth
  end function EmDee_coul_damped_smoothed

  type(c_ptr) function EmDee_coul_damped_square_smoothed( damp, skinWidth ) bind(C,name="EmDee_coul_damped_square_smoothed")
    import
    real(c_double), value :: damp
    real(c_double), value :: skinWidth
  end function EmDee_coul_damped_square_smoothed

  type(c_ptr) function EmDee_coul_square_smoothed( skinWidth ) bind(C,name="EmDee_coul_square_smoothed")
    import
    real(c_double), value :: skinWidth
  end function EmDee_coul_square_smoothed

  type(c_ptr) function EmDee_coul_shifted_square_smoothed( skinWidth ) bind(C,name="EmDee_coul_shifted_square_smoothed")
    import
    real(c_double), value :: skinWidth
  end function EmDee_coul_shifted_square_smoothed

  type(c_ptr) function EmDee_coul_long(  ) bind(C,name="EmDee_coul_long")
    import
  end function EmDee_coul_long

  type(c_ptr) function EmDee_kspace_ewald( accuracy ) bind(C,name="EmDee_kspace_ewald")
    import
    real(c_double), value :: accuracy
  end function EmDee_kspace_ewald

  type(c_ptr) function EmDee_bond_harmonic( k, r0 ) bind(C,name="EmDee_bond_harmonic")
    import
    real(c_double), value :: k
    real(c_double), value :: r0
  end function EmDee_bond_harmonic

  type(c_ptr) function EmDee_angle_harmonic( k, theta0 ) bind(C,name="EmDee_angle_harmonic")
    import
    real(c_double), value :: k
    real(c_double), value :: theta0
  end function EmDee_angle_harmonic

end interface

end module EmDee
