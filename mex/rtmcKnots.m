function K = rtmcKnots(material)
%RTMCKNOTS  The inverse-CDF knots of material.invcdf for rtmc_mex: a 1x1 cell (acoustics)
%   or a 2x2 cell {old mode, new mode} (elastics) of [cdf theta] matrices, read from the
%   griddedInterpolant objects MaterialClass.prepareSigmaOne builds (MaterialClass.m:2462).
if material.acoustics
    K = {pairOf(material.invcdf)};
else
    K = cell(2);
    for i = 1:2
        for j = 1:2
            K{i, j} = pairOf(material.invcdf{i, j});
        end
    end
end
end

function M = pairOf(F)
M = [F.GridVectors{1}(:) F.Values(:)];
end
