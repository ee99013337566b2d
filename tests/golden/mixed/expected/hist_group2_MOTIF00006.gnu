set output "hist_group2_MOTIF00006.ps"
set key autotitle columnhead
set terminal postscript landscape
set terminal postscript noenhanced
set xrange [-64.5106:21.597]
set yrange [0:166124]
set xlabel 'PWM score'
set ylabel 'count'
plot "hist_group2_MOTIF00006.dat" using 1:2 title 'MOTIF00006 (group2)' with boxes
