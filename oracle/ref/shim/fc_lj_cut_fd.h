/* ORACLE harness shim (project code): intentionally empty.  The real header
 * registers a force-constant style that needs a LAMMPS pair style at run
 * time; leaving it out drops only that registration. */
