function obs = radiativeTransfer(geometry, source, material, observation, opts)
%RADIATIVETRANSFER  Drop-in for the reference's radiativeTransfer with the particle loop
%   on the GPU: obs = radiativeTransfer(geometry, source, material, observation).
%   The set-up (radiativeTransfer.m:4-38) and the energy normalisation
%   (radiativeTransfer.m:160-191) are the reference's; the packet x time loop
%   (radiativeTransfer.m:40-158) is one call of the rtmc_mex gateway, which runs
%   initializeParticle, propagateParticleSmallDt / propagateParticle and observeTime for
%   every particle on the GPU and returns the uint32 histogram E.
%   opts (optional): see rtmcProblem (precision, seed, hist_shift, max_events).
%   Put this file, rtmc_mex, rtmcProblem, rtmcKnots and rtmcEdges ahead of the reference
%   on the MATLAB path.
if nargin < 5, opts = struct(); end
d = geometry.dimension;
if ~isfield(geometry, 'frame'), geometry.frame = 'spherical'; end
if ~material.acoustics && isprop(material, 'Q') && isscalar(material.Q) && isfinite(material.Q)
    warning(['Only one quality factor was provided for an elastic simulation. ', ...
             'The same value Q = %g will be used for both P and S waves.'], material.Q);
end

% particles: rounded up to whole packets of 1e5, as the reference counts them
Npk = 1e5;
N = ceil(source.numberParticles / Npk) * Npk;
[obs, E0, ~, ibins, ~, ~, ~, d1, d2] = initializeObservation(geometry, material.acoustics, observation, N);
material = MaterialClass.prepareSigma(material, d);

P = rtmcProblem(geometry, source, material, obs, ibins, opts);
E = reshape(rtmc_mex('forward', P, rtmcKnots(material), rtmcEdges(obs)), size(E0));

% energy density over [x1 x2 t (mode)]: counts over bin weights and N, then the factor of
% the integrated axes for the binned pair (radiativeTransfer.m:160-188)
obs.energyDensity = double(E) ./ (d1' * (d2 * obs.N));
key = sprintf('%d%d', ibins(1), ibins(2));
if obs.d == 3
    switch key
        case '12', obs.energyDensity = obs.energyDensity / obs.dz;
        case '13', obs.energyDensity = obs.energyDensity / obs.dy;
        case '23', obs.energyDensity = obs.energyDensity / obs.dx;
        case '14', obs.energyDensity = obs.energyDensity .* obs.dpsi / (obs.dy * obs.dz);
        case '24', obs.energyDensity = obs.energyDensity .* obs.dpsi / (obs.dx * obs.dz);
        case '34', obs.energyDensity = obs.energyDensity .* obs.dpsi / (obs.dx * obs.dy);
        otherwise, error('Unsupported bin combination in 3D');
    end
else
    switch key
        case '12'
        case '14', obs.energyDensity = obs.energyDensity .* obs.dpsi / obs.dy;
        case '24', obs.energyDensity = obs.energyDensity .* obs.dpsi / obs.dx;
        otherwise, error('Unsupported bin combination in 2D');
    end
end

% energy over time (radiativeTransfer.m:191)
obs.energy = squeeze(sum(sum(double(E), 1), 2)) / obs.N;
end
