-- self-gravitating blobs with a fixed timestep and mixed boundaries
solverName = 'EulerHLL'
integratorName = 'RungeKutta4_3_8thsRule'
size = {96, 64}
xmin = {-1.5, -1}
xmax = {1.5, 1}
boundaryMethods = {
	{min = 'PERIODIC', max = 'PERIODIC'},
	{min = 'MIRROR', max = 'FREEFLOW'},
	{min = 'NONE', max = 'NONE'},
}
useFixedDT = true
fixedDT = 2.5e-4
useGravity = true
gaussSeidelMaxIter = 0x10
defs = {
	idealGas_heatCapacityRatio = 7 / 5,
	selfGrav_gravitationalConstant = 4 * math.pi * 1e-1,
}
