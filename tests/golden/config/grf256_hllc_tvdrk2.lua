-- 3D log-normal density run: EulerHLLC, TVD-RK2, mirror walls on the unit cube
solverName = "EulerHLLC"
integratorName = "RungeKutta2TVD"
slopeLimiter = "VanLeer"      -- has no effect on the HLLC flux
size = {256, 256, 256}
xmin = {0, 0, 0}
xmax = {1, 1, 1}
cfl = .4
walls = {min = 'MIRROR', max = 'MIRROR'}
boundaryMethods = {walls, walls, walls}
defs = {}
defs.idealGas_heatCapacityRatio = 5/3
defs['selfGrav_gravitationalConstant'] = 2 ^ -1
