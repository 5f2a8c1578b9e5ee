"""Drop-in for the reference's per-particle data writer (LIBRARIES/LIBRARY_Write_particle_data.py:3-13):
one tab-separated ``<filename><particle_id>.dat`` per particle, a header at step 0, then one line per
call with the centre, the velocity (|vz|, as the reference writes it) and the normal, spring and
damping forces."""
from __future__ import annotations


def Particle_data_writer(particle, filename, timestep):
    path = filename + str(particle.particle_id) + ".dat"
    with open(path, "w" if timestep == 0 else "a") as f_out:
        if timestep == 0:
            f_out.write("Timestep\t Cm_x\t Cm_y\t Cm_z\t vx\t vy\t vz\t fx\t fy\t fz\t fsx\t fsy\t fsz\t fdx\t fdy\t fdz\n")
        c, v = particle.center_of_mass, particle.velocity
        fn, fs, fd = particle.force_normal, particle.force_n_spring, particle.force_n_damping
        vals = [timestep, c[0], c[1], c[2], v[0], v[1], abs(v[2]), fn[0], fn[1], fn[2], fs[0], fs[1], fs[2],
                fd[0], fd[1], fd[2]]
        f_out.write("\t".join(str(x) for x in vals) + "\n")
