-- Kelvin-Helmholtz benchmark run: EulerRoe, RK4, minmod, periodic 2048^2
-- (settings only; a file in the style the reference host reads)

--slopeLimiterName = 'Superbee'
slopeLimiter = 'MinMod'

--integratorName = 'ForwardEuler'
integratorName = 'RungeKutta4'

xmin = {-.5, -.5, -.5}
xmax = {.5, .5, .5}
useFixedDT = false
fixedDT = .001
cfl = .5
showTimestep = false

boundaryMethods = {
	{min='PERIODIC', max='PERIODIC'},
	{min='PERIODIC', max='PERIODIC'},
	{min='PERIODIC', max='PERIODIC'},
}

useGravity = false
gaussSeidelMaxIter = 20

defs = {
	idealGas_heatCapacityRatio = 1.4,
	selfGrav_gravitationalConstant = 1,
	srhd_solvePrimStopEpsilon = 1e-7,	-- read by other solvers only
	srhd_rhoMax = 1e+20,
}

camera = {}
heatMap = {enabled = true, variable = 'DENSITY', scale = 4, useLog = true, alpha = 1}
vectorField = {
	enabled = false;
	resolution = 64;
	scale = 1/8;
}

--[[ 3D
size = {64, 64, 64}
vectorField.resolution = 16
--]]
-- [[ 2D
N = 2048
size = {N, N}
--]]
--[==[ 1D
size = {1024}
]==]

solverName = 'EulerRoe'
