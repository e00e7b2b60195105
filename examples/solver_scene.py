"""A scene written against the reference's Solver / EntityFactory API
(src/core/lib.zig:13-130), stepped on the GPU through resolve2d_gb300.solver:
the same names, options and handles as the Zig source."""

from resolve2d_gb300.solver import (BodyOptions, Density, DiscOptions, Mass, Parameters,
                                    RectangleOptions, Solver)

solver = Solver.init(4.0, 2)                  # Solver.init(alloc, 4.0, 2)
fac = solver.entityFactory()
fac.makeDownwardsGravity(9.81)
ground = fac.makeRectangleBody(BodyOptions(pos=(0, -5), mass_prop=Density(5)),
                               RectangleOptions(width=200, height=10))
ground.body_unwrap().static = True
a = fac.makeDiscBody(BodyOptions(pos=(0, 4), mass_prop=Mass(2), mu=0.3), DiscOptions(radius=0.5))
b = fac.makeRectangleBody(BodyOptions(pos=(1.5, 4), mass_prop=Density(1)), RectangleOptions(1, 1))
fac.makeDistanceJoint(Parameters(beta=10), a, b, 1.5)
for _ in range(600):
    solver.process(1 / 60, 1, 8)              # InvalidRigidBodyId if a joint's body was removed
print(a.body_unwrap().props.pos)              # read back from the device on demand
solver.removeRigidBody(b.id)                  # swapRemove, as the reference
