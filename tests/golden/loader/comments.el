# comment line
% another

0 1
1 2
 2 3
2	0
