! refdriver.f90 -- test infrastructure for the translated reference.
!
! Driver entry points of this project (not reference code), translated to C
! by oracle/f90c.py together with the reference's own routines.  They set up
! what the reference's initialisation would (the species table of
! ModRamSpecies, src/ModRamInit.f90:47-64) so that the harness in
! oracle/refrun.py can call ram_run (src/ModRamRun.f90:16-225) directly.
module RefDriver

  implicit none

contains

  ! species(1:n) allocated and RAMSpecies defined (src/ModRamSpecies.f90)
  subroutine refdrv_species_begin(n)
    use ModRamVariables, only: species
    use ModRamSpecies,   only: DefineSpecies
    integer, intent(in) :: n
    if (allocated(species)) deallocate(species)
    allocate(species(n))
    call DefineSpecies
  end subroutine refdrv_species_begin

  ! species(i) = RAMSpecies(iS); wave-particle and EMIC processes off (the
  ! WPI/EMIC blocks of ram_run and ANISCH are outside the kinetic step)
  subroutine refdrv_species_set(i, iS)
    use ModRamVariables, only: species
    use ModRamSpecies,   only: RAMSpecies
    integer, intent(in) :: i, iS
    species(i) = RAMSpecies(iS)
    species(i)%WPI = .false.
    species(i)%EMIC = .false.
  end subroutine refdrv_species_set

  ! the charge of species(i), for the harness's checks
  subroutine refdrv_species_charge(i, q)
    use ModRamVariables, only: species
    integer, intent(in) :: i
    integer, intent(inout) :: q
    q = species(i)%s_charge
  end subroutine refdrv_species_charge

end module RefDriver
