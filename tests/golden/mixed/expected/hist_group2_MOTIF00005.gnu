set output "hist_group2_MOTIF00005.ps"
set key autotitle columnhead
set terminal postscript landscape
set terminal postscript noenhanced
set xrange [-51.3723:13.6733]
set yrange [0:132113]
set xlabel 'PWM score'
set ylabel 'count'
plot "hist_group2_MOTIF00005.dat" using 1:2 title 'MOTIF00005 (group2)' with boxes
