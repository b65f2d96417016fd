"""Enumerations of axes, cuboid faces/edges/corners, phases, flow regimes,
collision operators and boundary conditions, with the reference's values
(jyulb/defs.pxd:17-103).  The precision modes are additions of this engine.
"""
# Cartesian axes
X = 0
Y = 1
Z = 2

# cuboid faces: 1X has outward normal (-1,0,0), X1 has (1,0,0), etc.
FACE_1X = 0
FACE_X1 = 1
FACE_1Y = 2
FACE_Y1 = 3
FACE_1Z = 4
FACE_Z1 = 5

# cuboid edges
EDGE_1X_1Y = 0
EDGE_1X_Y1 = 1
EDGE_X1_1Y = 2
EDGE_X1_Y1 = 3
EDGE_1X_1Z = 4
EDGE_1X_Z1 = 5
EDGE_X1_1Z = 6
EDGE_X1_Z1 = 7
EDGE_1Y_1Z = 8
EDGE_1Y_Z1 = 9
EDGE_Y1_1Z = 10
EDGE_Y1_Z1 = 11

# cuboid corners
CORNER_1X_1Y_1Z = 0
CORNER_1X_1Y_Z1 = 1
CORNER_1X_Y1_1Z = 2
CORNER_1X_Y1_Z1 = 3
CORNER_X1_1Y_1Z = 4
CORNER_X1_1Y_Z1 = 5
CORNER_X1_Y1_1Z = 6
CORNER_X1_Y1_Z1 = 7

# phases
SOLID = 0
FLUID = 1
LIQUID = 2
VAPOUR = 3

# flow regimes
STOKES = 0
LAMINAR = 1
TURBULENT = 2

# collision operators
BGK = 0
TRT = 1
REGULARIZATION = 2
RECURRENCE_REL = 3

# boundary conditions
WALL = 0        # immobile and adiabatic
PERIODIC = 1
FIXED_DEN = 2   # defines implicitly the boundary normal velocity
FIXED_VEL = 3   # defines implicitly the boundary density
SYMMETRIC = 4   # specular reflection

# population storage / arithmetic of the GPU time step (engine addition)
FP64 = 0        # FP64 storage and arithmetic, the reference's operation order
FP32 = 1        # FP32 storage of f - w, FP32 arithmetic
FP16 = 2        # FP16 storage of 2^12 (f/w - 1), FP32 arithmetic
FP64_FAST = 3   # FP64 storage and arithmetic, regrouped and FMA-contracted
                # (within 1e-12 relative of FP64, not bit for bit)
