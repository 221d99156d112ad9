function E = rtmcEdges(obs)
%RTMCEDGES  The bin edges {binX, binY, binZ, binPsi} of initializeObservation for
%   rtmc_mex, in the frame's coordinates (binZ already sin(elevation) in 3D spherical
%   frames, binPsi cos(directions) reversed in 3D, as initializeObservation.m stores them).
E = {obs.binX, obs.binY, obs.binZ, obs.binPsi};
end
