"""Site operators and two-site terms used with the BP energies.

Two-site terms are lists of (coefficient, O) meaning sum_t c_t O (x) O on every
edge.  Pauli Y (x) Y is real: Y = i J with J = [[0, -1], [1, 0]], so
Y (x) Y = -J (x) J."""
import numpy as np

SZ = np.array([[0.5, 0.0], [0.0, -0.5]])
SX = np.array([[0.0, 0.5], [0.5, 0.0]])
PX = np.array([[0.0, 1.0], [1.0, 0.0]])
PZ = np.array([[1.0, 0.0], [0.0, -1.0]])
PJ = np.array([[0.0, -1.0], [1.0, 0.0]])

# Heisenberg, J = 1, Pauli matrices: XX + YY + ZZ per edge
HEISENBERG = [(1.0, PX), (-1.0, PJ), (1.0, PZ)]
# Ising coupling -ZZ per edge
ISING_ZZ = [(-1.0, PZ)]
